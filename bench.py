#!/usr/bin/env python3
"""Benchmark of the GB300 prover backend.

Default workload (`--workload poseidon`): one proof of the Poseidon2 AIR with 2^16 rows (2^19
permutations, 1264 trace + 32 LogUp interaction columns), seeded uniform initial states,
PcsConfig { pow_bits 10, FriConfig(0, 1, 3) }. One step = one proof through the C ABI
(stwo_prove_poseidon). `value` is trace cells/s = 2^16 x 1296 / proof time with the initial
states resident in HBM; in `e2e` they stay in pinned host memory and the trace kernel reads them
across the host link inside the timed region (the proof bytes always come back to the host).
Per-stage device times come from one extra, separately timed proof. At one GPU with at least 3
steps, the line also carries `batch` and `serve`: the batch and served workloads below, run
after the timed region with fewer steps.

Kernel workload (`--workload kernels`): the kernel microbench on synthetic seeded inputs —
interpolate then evaluate 256 columns of 2^20 M31 words (canonic coset, log 20) at blowup 4
(2^22 points each), Blake2s Merkle commit over the 256 x 2^22 evaluations, and one FRI fold of a
2^22-point QM31 circle evaluation down to a 2^4 line with seeded alphas. One step = that whole
pass. Inputs (1 GiB) are larger than L2 (129 MB), so no explicit flush is needed between steps.

`value` is trace cells/s (256 x 2^20 input cells per step) with inputs resident in HBM when the
timed region starts; `e2e` is the same metric through the public C ABI with the inputs copied
from pinned host memory and the Merkle root + last FRI layer read back inside the timed region.

`--impl reference` times the oracle (C++ restatement of the reference CPU backend; the reference
Rust crate cannot be built without a Rust toolchain) on all host cores: for the Poseidon2
workload each step is one whole proof of the same 2^16-row configuration; the kernel workload
takes a bounded sample of its columns.
Multi-GPU (torchrun): independent replicas per rank, no collective on the data path.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

P = (1 << 31) - 1
GAMMA = 0x9E3779B97F4A7C15
MASK64 = (1 << 64) - 1


def gen_words(k: int, c: int, n: int):
    """Word i of column c of workload k: splitmix64(k + (c*2^32 + i + 1) * GAMMA) mod P."""
    import numpy as np

    i = np.arange(n, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = np.uint64(k) + (np.uint64(c << 32) + i + np.uint64(1)) * np.uint64(GAMMA)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z % np.uint64(P)).astype(np.uint32)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every `period_ms` (25 ms) during the timed
    region (a read-only query)."""

    def __init__(self, index: int, period_ms: int = 25):
        self.index = index
        self.period_ms = period_ms
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", str(self.period_ms)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for nm, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm), "period_ms": self.period_ms}


def autotune_pass(run_once):
    """One untimed run with the library's autotuner measuring the launch shapes of every size it
    meets (results unchanged), then the table in use for everything after."""
    from stwo_gb300 import autotune

    autotune.set_mode(autotune.TUNE)
    try:
        run_once()
    finally:
        autotune.set_mode(autotune.USE)
    return {"entries": len(autotune.entries()), "choices": autotune.summary(),
            "note": "launch shapes timed once per size before the warm-up, then used"}


def int_bound(kind, achieved, clocks, local):
    """Integer-datapath bound of a stage from the library's register-only probe of its inner
    operation (`kind` "butterfly" or "blake2s"): the probe's issue cost in SM cycles per warp-wide
    operation, times 4 schedulers x SMs x the SM clock sampled during the timed region."""
    import torch

    from stwo_gb300 import _lib

    rate, cyc, pmhz = C.c_double(), C.c_double(), C.c_double()
    fn, rounds = {"butterfly": ("stwo_butterfly_rate", 512), "blake2s": ("stwo_blake2s_rate", 256)}[kind]
    _lib.call(fn, rounds, C.byref(rate), C.byref(cyc), C.byref(pmhz), None)
    csum = clocks or {}
    mhz = csum.get("sm_mhz") or csum.get("sm_max_mhz") or 2070.0
    n_sm = torch.cuda.get_device_properties(local).multi_processor_count
    bound = 4 * n_sm * mhz * 1e6 * 32 / cyc.value
    unit = {"butterfly": "butterflies/s", "blake2s": "compressions/s"}[kind]
    return {"unit": unit, "achieved": achieved, "peak": bound, "frac": achieved / bound,
            "cycles_per_warp_op": cyc.value, "sm_mhz": mhz, "sms": n_sm,
            "probe_rate_event_timed": rate.value, "probe_sm_mhz": pmhz.value,
            "peak_source": f"{fn}: the library's {kind} with every operand in registers, one full wave of "
                           "blocks; its issue cost in SM cycles (clock64 per block) x 4 schedulers x SMs x "
                           "the SM clock sampled during the timed region"}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# --------------------------------------------------------------------------- kernel microbench
class KernelsWorkload:
    N_COLS, LOG, BLOWUP, FRI_LOG, FRI_LAST = 256, 20, 2, 22, 4

    def __init__(self, n_cols=None):
        import numpy as np
        import torch

        from stwo_gb300 import _lib
        from stwo_gb300.backend import CudaBackend, SecureColumn, TwiddleTree
        from stwo_gb300.circle import canonic_half_coset

        self.B, self.SC = CudaBackend, SecureColumn
        if n_cols:
            self.N_COLS = n_cols
        L = self.LOG + self.BLOWUP
        self.L = L
        n, N = 1 << self.LOG, 1 << L
        self.host_in = torch.empty((self.N_COLS, n), dtype=torch.int32).pin_memory()
        hv = self.host_in.numpy().view(np.uint32)
        for c in range(self.N_COLS):
            hv[c] = gen_words(1, c, n)
        self.inp = self.host_in.cuda()
        self.work = torch.empty_like(self.inp)
        self.evals = torch.empty((self.N_COLS, N), dtype=torch.int32, device="cuda")
        self.tw = TwiddleTree(canonic_half_coset(L))
        self.small, self.big = canonic_half_coset(self.LOG), canonic_half_coset(L)
        self.fri_half = canonic_half_coset(self.FRI_LOG)
        self.fri_tw = self.tw if self.FRI_LOG <= L else TwiddleTree(self.fri_half)
        self.fsrc = SecureColumn([torch.from_numpy(gen_words(1, 1000 + k, 1 << self.FRI_LOG).view(np.int32)).cuda()
                                  for k in range(4)])
        self.alphas = [tuple(int(x) for x in gen_words(1, 2000, 4 * self.FRI_LOG)[4 * j:4 * j + 4])
                       for j in range(self.FRI_LOG)]
        self.layers = [torch.empty(((1 << lg), 8), dtype=torch.int32, device="cuda") for lg in range(L + 1)]
        self.line = SecureColumn([torch.empty(1 << (self.FRI_LOG - 1), dtype=torch.int32, device="cuda")
                                  for _ in range(4)])
        self.work_cols = [self.work[c] for c in range(self.N_COLS)]
        self.eval_cols = [self.evals[c] for c in range(self.N_COLS)]
        self.cells = self.N_COLS * n
        self.root_host = torch.empty(8, dtype=torch.int32).pin_memory()
        self.fri_host = torch.empty((4, 1 << self.FRI_LAST), dtype=torch.int32).pin_memory()
        self.lib = _lib.load()

    def restore(self):
        self.work.copy_(self.inp)

    def stages(self, ev=None):
        """The hot path; `ev` (list of CUDA events) brackets interpolate / evaluate / merkle / fri."""
        import torch

        from stwo_gb300.circle import double

        B = self.B
        mark = (lambda i: ev[i].record()) if ev else (lambda i: None)
        mark(0)
        B.interpolate_columns(self.work_cols, self.small, self.tw)
        mark(1)
        B.evaluate_polynomials(self.work_cols, self.big, self.tw, out=self.eval_cols)
        mark(2)
        B.commit_on_layer(self.L, None, self.eval_cols, out=self.layers[self.L])
        mark(3)
        for lg in range(self.L - 1, -1, -1):
            B.commit_on_layer(lg, self.layers[lg + 1], [], out=self.layers[lg])
        mark(4)
        for c in self.line.cols:
            c.zero_()
        B.fold_circle_into_line(self.line, self.fsrc, self.fri_half, self.alphas[0], self.fri_tw)
        cur, dom = self.line, self.fri_half
        j = 1
        while len(cur) > (1 << self.FRI_LAST):
            cur = B.fold_line(cur, dom, self.alphas[j], self.fri_tw)
            dom = double(dom)
            j += 1
        self.last = cur
        mark(5)
        del torch

    def readback(self):
        self.root_host.copy_(self.layers[0][0], non_blocking=True)
        for k in range(4):
            self.fri_host[k].copy_(self.last.cols[k], non_blocking=True)


class PoseidonWorkload:
    """Single proof of the Poseidon2 AIR: 2^16 rows x 8 permutations (2^19 permutations), seeded
    uniform initial states, LogUp interaction trace, pow_bits 10, blowup 2, 3 FRI queries."""

    LOG = 16
    CFG = (10, 1, 0, 3)
    TRACE_COLS = 1264 + 32

    def __init__(self, log=None):
        import numpy as np
        import torch

        if log:
            self.LOG = log
        n = (1 << self.LOG) * 8 * 16
        self.host_in = torch.empty(n, dtype=torch.int32).pin_memory()
        self.host_in.numpy().view(np.uint32)[:] = gen_words(3, 0, n)
        self.inp = self.host_in.cuda()
        self.work = torch.empty_like(self.inp)
        self.cells = (1 << self.LOG) * self.TRACE_COLS

    def step(self, from_host=False):
        """One proof. from_host: the initial states stay in pinned host memory and the trace
        kernel reads them across the host link inside the proof (no staging copy)."""
        from stwo_gb300.prover import prove_poseidon

        src = self.host_in if from_host else self.inp
        self.proof, self.claimed_sum = prove_poseidon(self.LOG, src, self.CFG)
        return self.proof

    # DRAM bytes (read + write) of the composition extension's kernels in one proof of 2^14 rows,
    # from an ncu capture (dram__bytes_read.sum + dram__bytes_write.sum); traffic grows with the rows.
    COMPOSITION_EXT_TRAFFIC_2E14 = 836.6e6

    def stage_traffic(self):
        """Measured DRAM traffic of the stages that have an ncu capture, scaled to 2^LOG rows."""
        return {"Composition extension": self.COMPOSITION_EXT_TRAFFIC_2E14 * (1 << self.LOG) / (1 << 14)}

    def stage_bytes(self):
        """Algorithmic HBM bytes of the HBM-bound stages (reads + writes of the column data)."""
        n = 1 << self.LOG
        cols = self.TRACE_COLS
        return {
            "Composition extension": cols * (4 * n + 4 * 4 * n),
            "Constraint point-wise eval": cols * 4 * 4 * n + 4 * 4 * 4 * n,
            "Interpolation for commitment": cols * 8 * n,
            "Compute FRI quotients": cols * 4 * n + 4 * 4 * 2 * n + 4 * 4 * 8 * n,
        }


class GkrWorkload:
    """GKR batch proof (gkr_prover::prove_batch) of one LogUp-generic input layer of 2^20 leaves: the
    shape of the Poseidon2 relation at 2^16 rows (8 permutations x 2 fractions per row), with
    seeded uniform QM31 numerators and denominators. One step = one prove_batch through the C ABI
    (stwo_gkr_prove_batch) from a default channel."""

    LOG = 20

    def __init__(self, log=None):
        import numpy as np
        import torch

        from stwo_gb300 import _lib

        if log:
            self.LOG = log
        n = 1 << self.LOG
        self.host_in = torch.empty(8 * n, dtype=torch.int32).pin_memory()
        self.host_in.numpy().view(np.uint32)[:] = gen_words(6, 0, 8 * n)
        self.dev = self.host_in.cuda()
        self.work = torch.empty_like(self.dev)
        self.cap = 1 << 20
        self.out = (C.c_uint8 * self.cap)()
        self.len = C.c_size_t()
        self.lib = _lib

    def _ptrs(self, t):
        n = 1 << self.LOG
        base = t.data_ptr()
        nums = (C.c_void_p * 4)(*[base + 4 * c * n for c in range(4)])
        dens = (C.c_void_p * 4)(*[base + 4 * (4 + c) * n for c in range(4)])
        return nums, dens

    def step(self, from_host=False):
        import torch

        src = self.work if from_host else self.dev
        if from_host:
            self.work.copy_(self.host_in, non_blocking=True)
        nums, dens = self._ptrs(src)
        kinds = (C.c_uint32 * 1)(1)
        logs = (C.c_uint32 * 1)(self.LOG)
        self.lib.call("stwo_gkr_prove_batch", 1, kinds, logs, nums, dens, None, self.out, self.cap,
                      C.byref(self.len), None, C.c_void_p(torch.cuda.current_stream().cuda_stream))
        return bytes(self.out[:self.len.value])

    def algorithmic_bytes(self):
        """Compulsory HBM bytes of one proof: building the circuit (each next_layer reads 2m gates
        and writes m, 32 B per gate) and every sum-check round (the first round of a layer reads
        its 2^k gates; later rounds read the previous 2m folded gates and write m; plus the eq
        evaluations each round reads and the per-layer eq table writes)."""
        total = 0
        for k in range(self.LOG, 0, -1):
            total += 32 * (1 << k) + 32 * (1 << (k - 1))
        for k in range(1, self.LOG + 1):  # oracle over the layer with k variables
            total += 16 * (1 << max(k - 2, 0))  # eq table of 2^(k-2) written
            cur = 1 << k
            total += 32 * cur + 16 * (cur // 4)
            while cur > 2:
                cur //= 2
                total += 32 * 2 * cur + 32 * cur + (16 * (cur // 4) if cur >= 4 else 0)
        return total


def run_gkr(args, world, rank, local, lib, barrier, max_over_ranks):
    import numpy as np
    import torch

    wl = GkrWorkload()
    # The input (32 MiB) fits in L2, so L2 is flushed by a 256 MiB write before every timed step.
    flush = torch.empty(64 << 20, dtype=torch.int32, device="cuda")
    for _ in range(args.warmup):
        wl.step()
    barrier()
    launches0 = lib.stwo_kernel_launches()
    times = []
    with ClockSampler(local) as clk:
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            proof = wl.step()
            e1.record()
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        barrier()
        wall = time.perf_counter() - t0
    launches = lib.stwo_kernel_launches() - launches0
    step_ms = max_over_ranks(float(np.mean(times)))
    for _ in range(max(1, args.warmup // 2)):
        wl.step(from_host=True)
    barrier()
    et = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        wl.step(from_host=True)
        torch.cuda.synchronize()
        et.append((time.perf_counter() - t1) * 1e3)
    e2e_ms = max_over_ranks(float(np.mean(et)))
    if rank != 0:
        return
    peak, peak_kind = measured_peaks()
    leaves = 1 << wl.LOG
    ab = wl.algorithmic_bytes()
    ach = ab / (step_ms / 1e3) / 1e9
    line = {
        "metric": "GKR prove_batch leaves/s (LogUp generic, 2^20 leaves)",
        "value": leaves * world / (step_ms / 1e3),
        "unit": "leaves/s",
        "proof_s": step_ms / 1e3,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32 (QM31 as 4 M31 words)",
        "data": "synthetic: seeded uniform QM31 numerators and denominators (splitmix64 mod P)",
        "config": {"workload": "GKR batch proof, one LogUp-generic layer of 2^20 leaves (Poseidon2 relation shape "
                               "at 2^16 rows)", "log_leaves": wl.LOG,
                   "l2": "input (32 MiB) fits in L2: flushed by a 256 MiB write before each timed step",
                   "parallelism": f"replicas x{world}"},
        "proof_bytes": len(proof),
        "roofline": {"bound": "hbm", "kernel": "whole prove_batch (latency-bound: one host round trip per "
                                               "sum-check round)", "achieved": ach, "peak": peak, "unit": "GB/s",
                     "frac": ach / peak, "peak_kind": peak_kind, "traffic": None,
                     "algorithmic_bytes_per_launch": ab},
        "e2e": {"value": leaves * world / (e2e_ms / 1e3), "unit": "leaves/s", "proof_s": e2e_ms / 1e3,
                "h2d_bytes_per_step": 32 * leaves, "d2h_bytes_per_step": len(proof)},
        "gpu_launches": int(launches),
        "wall_s": wall,
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline and world == 1:  # the CPU baseline is timed at N=1 only
        line["cpu_baseline"] = cpu_baseline_gkr(args.cpu_threads)
    print(json.dumps(line), flush=True)


def cpu_baseline_gkr(threads=0, log=20):
    """The oracle's GKR batch proof (OpenMP on all host cores) of the same 2^20-leaf layer."""
    import numpy as np

    import oracle.pyoracle as O

    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    nthreads = threads or os.cpu_count() or 1
    n = 1 << log
    w = gen_words(6, 0, 8 * n).reshape(8, n)
    layers = [(O.LOGUP_GENERIC, [np.ascontiguousarray(w[:4]), np.ascontiguousarray(w[4:])])]
    t0 = time.perf_counter()
    O.gkr_prove(layers)
    secs = time.perf_counter() - t0
    return {"value": n / secs, "unit": "leaves/s", "cores": nthreads, "kind": "port", "proof_s": secs,
            "sample": f"one full GKR batch proof of the same 2^{log}-leaf layer: {secs:.2f} s"}


class BatchWorkload:
    """Mixed batch of whole proofs: n jobs, half wide-Fibonacci (100 columns, 2^log rows) and half
    Poseidon2 (2^log instances = 2^(log-3) rows), log sizes uniform in [lo, hi] from `seed`, each
    with its seeded inputs resident in HBM. Wide-Fibonacci uses PcsConfig::default(); Poseidon2
    pow_bits 10. With arrivals (the served workload) the AIR of each request is uniform over
    wide-Fibonacci, Poseidon2 and the Blake2s round AIR (2^log rows of one BLAKE2s round each,
    uniform 32-bit state and message words, PcsConfig::default())."""

    def __init__(self, n=64, lo=10, hi=18, seed=4, arrivals=None):
        import numpy as np
        import torch

        from stwo_gb300.prover import AIR_BLAKE_ROUND, AIR_POSEIDON, AIR_WIDE_FIB

        rng = np.random.default_rng(seed)
        if arrivals is None:
            airs = rng.permutation([AIR_WIDE_FIB] * (n // 2) + [AIR_POSEIDON] * (n - n // 2))
        else:
            airs = rng.integers(0, 3, n)
        logs = rng.integers(lo, hi + 1, n)
        self.arrivals = arrivals
        self.specs = []
        self.host = []
        for i, (air, log) in enumerate(zip(airs, logs)):
            if air == AIR_WIDE_FIB:
                rows = int(log)
                words = gen_words(40 + seed, i, 2 << rows)
                cfg, cols = (5, 1, 0, 3), 100
            elif air == AIR_BLAKE_ROUND:
                rows = int(log)
                words = np.random.default_rng((seed, i)).integers(0, 2**32, (1 << rows) * 32, dtype=np.uint64)
                words = words.astype(np.uint32)
                cfg, cols = (5, 1, 0, 3), 0
            else:
                rows = int(log) - 3
                words = gen_words(40 + seed, i, (1 << rows) * 128)
                cfg, cols = (10, 1, 0, 3), 0
            h = torch.empty(len(words), dtype=torch.int32).pin_memory()
            h.numpy().view(np.uint32)[:] = words
            self.host.append(h)
            self.specs.append((int(air), rows, cols, cfg))
        self.dev = [h.cuda() for h in self.host]
        cells_per_row = {AIR_WIDE_FIB: None, AIR_POSEIDON: 1296, AIR_BLAKE_ROUND: 384 + 260}
        self.cells = sum((1 << r) * (c if a == AIR_WIDE_FIB else cells_per_row[a]) for a, r, c, _ in self.specs)

    def jobs(self, from_host=False):
        from stwo_gb300.prover import AIR_WIDE_FIB, Job

        if from_host:
            for d, h in zip(self.dev, self.host):
                d.copy_(h, non_blocking=True)
        out = []
        for (air, rows, cols, cfg), d in zip(self.specs, self.dev):
            if air == AIR_WIDE_FIB:
                n = 1 << rows
                out.append(Job(air, rows, cfg, n_cols=cols, a=d[:n], b=d[n:]))
            else:
                out.append(Job(air, rows, cfg, init=d))
        return out


def run_batch(args, world, rank, local, lib, barrier, max_over_ranks, emit=True):
    """Batched proofs/s of 64 mixed proofs on a worker pool, beside the same jobs one at a time.
    With emit=False the JSON line is returned instead of printed."""
    import numpy as np
    import torch

    from stwo_gb300.prover import prove_batch

    wl = BatchWorkload()
    workers = args.workers or 16  # on GB300: 8 workers 38.7 ms per batch, 12: 37.7, 16: 38.0, 24: 40.9

    def run(n_workers, from_host=False):
        jobs = wl.jobs(from_host)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = prove_batch(jobs, n_workers=n_workers)
        torch.cuda.synchronize()
        return time.perf_counter() - t0, res

    tuned = autotune_pass(lambda: run(1))  # one worker: each shape timed with the GPU to itself
    for _ in range(args.warmup):
        run(workers)
    barrier()
    launches0 = lib.stwo_kernel_launches()
    with ClockSampler(local) as clk:
        ts = [run(workers)[0] for _ in range(args.steps)]
    launches = lib.stwo_kernel_launches() - launches0
    step_s = max_over_ranks(float(np.mean(ts)))
    # Plain mode is the median of three runs: one run alone is exposed to host-side hiccups.
    plains = [run(1) for _ in range(3)]
    plain_s, plain_res = sorted(plains, key=lambda x: x[0])[1]
    e2e_s = float(np.mean([run(workers, from_host=True)[0] for _ in range(max(1, args.steps // 2))]))
    _, res = run(workers)
    same = all(a.proof == b.proof for a, b in zip(res, plain_res))
    if rank != 0:
        return
    n = len(wl.specs)
    lat = sorted(r.latency_ms for r in res)
    line = {
        "metric": "batched proofs/s (64 mixed wide-Fibonacci / Poseidon2 proofs, log sizes 10..18)",
        "value": n * world / step_s, "unit": "proofs/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32 (M31 field words)",
        "data": "synthetic: seeded inputs (splitmix64 mod P), sizes from seed 4",
        "config": {"workload": "64 proofs: 32 wide-Fibonacci (100 cols, 2^10..2^18 rows, PcsConfig default) + "
                               "32 Poseidon2 (2^10..2^18 instances, pow 10)", "workers": workers,
                   "trace_cells_per_batch": wl.cells,
                   "l2": "working set (GBs) larger than L2; no flush", "timing": "host wall clock around the "
                   "synchronous batch call (every stream complete at return)", "parallelism": f"replicas x{world}"},
        "plain": {"value": n / plain_s, "unit": "proofs/s", "ms": plain_s * 1e3,
                  "runs_ms": [round(t * 1e3, 3) for t, _ in plains],
                  "note": "the same jobs one at a time (one worker)"},
        "speedup_vs_plain": plain_s / step_s,
        # Where plain mode's time goes: the proofs whose solo run is long enough to fill the GPU,
        # and the rest (latency-bound chains of short kernels that batching overlaps).
        "plain_breakdown": {
            "solo_ms_of_jobs_over_1ms": round(sum(r.run_ms for r in plain_res if r.run_ms >= 1.0), 3),
            "jobs_over_1ms": sum(1 for r in plain_res if r.run_ms >= 1.0),
            "solo_ms_of_other_jobs": round(sum(r.run_ms for r in plain_res if r.run_ms < 1.0), 3)},
        "proofs_identical_to_plain": same,
        "trace_cells_per_s": wl.cells * world / step_s,
        "latency_ms_in_batch": {"p50": lat[len(lat) // 2], "p99": lat[min(len(lat) - 1, int(0.99 * len(lat)))]},
        "e2e": {"value": n * world / e2e_s, "unit": "proofs/s", "ms": e2e_s * 1e3,
                "h2d_bytes_per_step": sum(h.numel() * 4 for h in wl.host),
                "d2h_bytes_per_step": sum(len(r.proof) for r in res)},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
        "autotune": tuned,
    }
    if not emit:
        return line
    print(json.dumps(line), flush=True)


def run_blake_round(args, world, rank, local, lib, barrier, max_over_ranks):
    """One proof of the Blake2s round AIR (BlakeRoundComponent alone): 2^log rows (default 16) of
    one BLAKE2s round each, uniform 32-bit state and message words, PcsConfig::default()."""
    import numpy as np
    import torch

    from stwo_gb300 import _lib
    from stwo_gb300.prover import prove_blake_round

    log = args.log_rows or 16
    cfg = (5, 1, 0, 3)
    n = (1 << log) * 32
    host = torch.empty(n, dtype=torch.int32).pin_memory()
    host.numpy().view(np.uint32)[:] = np.random.default_rng(11).integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    inp = host.cuda()
    cells = (1 << log) * (384 + 260)
    for _ in range(args.warmup):
        prove_blake_round(log, inp, cfg)
    barrier()
    launches0 = lib.stwo_kernel_launches()
    times = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            proof, _ = prove_blake_round(log, inp, cfg)
            e1.record()
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
    launches = lib.stwo_kernel_launches() - launches0
    step_ms = max_over_ranks(float(np.mean(times)))
    work = torch.empty_like(inp)
    et = []
    for _ in range(args.steps):
        t1 = time.perf_counter()
        work.copy_(host, non_blocking=True)
        prove_blake_round(log, work, cfg)
        torch.cuda.synchronize()
        et.append((time.perf_counter() - t1) * 1e3)
    e2e_ms = max_over_ranks(float(np.mean(et)))
    _lib.call("stwo_set_stage_timing", 1)
    prove_blake_round(log, inp, cfg)
    names = (C.c_char_p * 64)()
    ms = (C.c_float * 64)()
    k = lib.stwo_stage_times(names, ms, 64)
    _lib.call("stwo_set_stage_timing", 0)
    stages = {names[i].decode(): float(ms[i]) for i in range(min(k, 64)) if not names[i].decode().startswith("host")}
    if rank != 0:
        return
    line = {
        "metric": f"Blake2s round AIR proof s & trace cells/s (2^{log} rows)",
        "value": cells * world / (step_ms / 1e3), "unit": "trace cells/s", "proof_s": step_ms / 1e3,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32 (M31 field words)",
        "data": "synthetic: uniform 32-bit state and message words (seed 11)",
        "config": {"workload": f"Blake2s round AIR (BlakeRoundComponent alone), 2^{log} rows, 384 trace + 260 "
                               "interaction columns", "log_n_rows": log, "trace_cells": cells,
                   "pcs_config": list(cfg), "l2": "working set larger than L2; no flush",
                   "parallelism": f"replicas x{world}"},
        "proof_bytes": len(proof),
        "stages_ms": stages,
        "e2e": {"value": cells * world / (e2e_ms / 1e3), "unit": "trace cells/s", "proof_s": e2e_ms / 1e3,
                "h2d_bytes_per_step": n * 4, "d2h_bytes_per_step": len(proof)},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


def run_blake_full(args, world, rank, local, lib, barrier, max_over_ranks):
    """One proof of the reference's full Blake example (prove_blake: scheduler, two round
    components, five XOR tables over preprocessed XOR tables) for 2^log instances (default 10),
    PcsConfig::default(), on the per-operation path: trace generated in HBM, generated constraint
    and interaction kernels, backend operations through the C ABI. Step time is wall clock with the
    device synchronised (the path is driven from the host); the oracle's prove_blake on the host
    cores is timed beside it on the same configuration."""
    import numpy as np
    import torch

    from stwo_gb300 import framework_prover

    log = args.log_rows or 10
    cfg = (5, 1, 0, 3)
    n = 1 << log
    cells = n * (384 + 24) + 8 * n * (384 + 260) + 2 * n * (384 + 260) + sum(
        (1 << (2 * e)) * (1 << (2 * (w - e))) + 4 * ((1 << (2 * e)) + 1) // 2 * (1 << (2 * (w - e)))
        for w, e in ((12, 4), (9, 2), (8, 2), (7, 2), (4, 0)))
    for _ in range(max(args.warmup, 1)):
        proof, sums = framework_prover.prove_blake(log, cfg)
    barrier()
    launches0 = lib.stwo_kernel_launches()
    times = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            proof, sums = framework_prover.prove_blake(log, cfg)
            torch.cuda.synchronize()
            times.append((time.perf_counter() - t0) * 1e3)
    launches = (lib.stwo_kernel_launches() - launches0) // max(args.steps, 1)
    step_ms = max_over_ranks(float(np.median(times)))
    if rank != 0:
        return
    cpu = None
    if world == 1:
        from oracle import pyoracle
        from stwo_gb300.build import build_oracle

        build_oracle()
        t0 = time.perf_counter()
        want, want_sums = pyoracle.prove_blake(log, cfg)
        cpu_s = time.perf_counter() - t0
        assert want == proof and want_sums == sums, "device proof differs from the oracle's"
        cpu = {"value": n / cpu_s, "unit": "BLAKE2s instances/s", "proof_s": cpu_s, "cores": os.cpu_count(),
               "kind": "port", "sample": f"one whole prove_blake of 2^{log} instances (the same proof)"}
    line = {
        "metric": f"full Blake example proof s & BLAKE2s instances/s (2^{log} instances)",
        "value": n * world / (step_ms / 1e3), "unit": "BLAKE2s instances/s", "proof_s": step_ms / 1e3,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32 (M31 field words)",
        "data": "the example's own inputs (instance 16 r + l: state words r + 2l, message words r + 2l + 1)",
        "config": {"workload": f"prove_blake, 2^{log} instances: scheduler 2^{log}, rounds 2^{log + 3} and "
                               f"2^{log + 1} rows, XOR tables 12/4, 9/2, 8/2, 7/2, 4/0",
                   "log_instances": log, "trace_and_interaction_cells": cells, "pcs_config": list(cfg),
                   "path": "per-operation C ABI driven from Python (framework_prover.prove_blake)",
                   "l2": "no flush", "parallelism": f"replicas x{world}"},
        "proof_bytes": len(proof),
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)


def run_serve(args, world, rank, local, lib, barrier, max_over_ranks, emit=True):
    """Served proving: Poisson arrivals (rate 200/s, seed 5), AIR uniform over wide-Fibonacci,
    Poseidon2 and the Blake2s round AIR, log sizes 12..20, HBM budget 150 GB; latency percentiles
    beside a plain one-at-a-time server. With emit=False the JSON line is returned instead of
    printed."""
    import numpy as np
    import torch

    from stwo_gb300.prover import Server

    n_req = args.requests or 200
    rate = 200.0
    rng = np.random.default_rng(5)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n_req))
    wl = BatchWorkload(n=n_req, lo=12, hi=20, seed=5, arrivals=arrivals)
    workers = args.workers or 8
    budget = 150 << 30

    def serve(n_workers):
        jobs = wl.jobs()
        torch.cuda.synchronize()
        with Server(n_workers=n_workers, hbm_budget=budget) as srv:
            t0 = time.perf_counter()
            tickets = []
            for j, at in zip(jobs, arrivals):
                delay = t0 + at - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                tickets.append(srv.submit(j))
            res = [srv.wait(t) for t in tickets]
            wall = time.perf_counter() - t0
        return res, wall

    for _ in range(args.warmup):
        serve(workers)
    barrier()
    with ClockSampler(local) as clk:
        runs = [serve(workers) for _ in range(args.steps)]
    plain, plain_wall = serve(1)
    if rank != 0:
        return

    def pct(res, q):
        lat = sorted(r.latency_ms for r in res)
        return lat[min(len(lat) - 1, int(q * len(lat)))]

    p99 = float(np.median([pct(r, 0.99) for r, _ in runs]))
    p50 = float(np.median([pct(r, 0.50) for r, _ in runs]))
    same = all(a.proof == b.proof for a, b in zip(runs[-1][0], plain))
    line = {
        "metric": "served p99 latency vs plain (Poisson 200/s, wide-Fibonacci / Poseidon2 / Blake2s round, "
                  "log 12..20)",
        "value": p99, "unit": "ms (p99 latency)",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": float(np.mean([w for _, w in runs])) * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "u32 (M31 field words)",
        "data": "synthetic: Poisson arrivals and sizes from seed 5, seeded inputs (splitmix64 mod P)",
        "config": {"workload": f"{n_req} requests, Poisson rate 200/s, AIR uniform in {{wide-Fibonacci (100 cols), "
                               f"Poseidon2, Blake2s round (BlakeRoundComponent alone)}}, log size uniform 12..20, "
                               f"HBM budget 150 GB", "workers": workers,
                   "air_mix": {name: int(sum(1 for a, _, _, _ in wl.specs if a == k))
                               for k, name in ((0, "wide_fib"), (1, "poseidon2"), (2, "blake2s_round"))},
                   "l2": "working set larger than L2; no flush", "parallelism": f"replicas x{world}"},
        "p50_ms": p50,
        "plain": {"p99_ms": pct(plain, 0.99), "p50_ms": pct(plain, 0.50), "wall_s": plain_wall,
                  "note": "the same arrivals served one at a time (one worker)"},
        "p99_vs_plain": p99 / pct(plain, 0.99),
        "throughput_proofs_per_s": n_req / float(np.mean([w for _, w in runs])),
        "proofs_identical_to_plain": same,
        "e2e": {"value": p99, "unit": "ms (p99 latency)", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": sum(len(r.proof) for r in plain),
                "note": "inputs resident; proof bytes returned to the host per request"},
        "gpu_launches": None,
        "clocks": clk.summary(),
    }
    if not emit:
        return line
    print(json.dumps(line), flush=True)


def run_constraints(args, world, rank, local, lib, barrier, max_over_ranks):
    """Constraint point-wise evaluation (ComponentProver::evaluate_constraint_quotients_on_domain
    after its extension step) of one component per AIR, on seeded uniform column words resident
    in HBM: Poseidon2 at 2^16 rows (1,296 columns on 2^18 points) and, generated only, Plonk and
    the wide-Fibonacci AIR at 2^20 rows. One step = one call per AIR. The generated kernels
    (stwo_eval_constraints_codegen, compiled once with NVRTC before timing) are timed beside the
    hand-written ones (stwo_eval_constraints) where those exist; `value` is the generated
    Poseidon2 kernel's evaluation-domain rows/s."""
    import numpy as np
    import torch

    from stwo_gb300 import _lib, airs, codegen

    def rq(rng):
        return tuple(int(v) for v in rng.integers(0, P, 4))

    specs = [("poseidon", 16, 1), ("plonk", 20, None), ("wide_fib", 20, 0)]
    if args.log_rows:  # a smaller Poseidon2 case alone (profiling captures)
        specs = [("poseidon", args.log_rows, 1)]
    out = {}
    peak, peak_kind = measured_peaks()
    for name, log, hand_id in specs:
        rng = np.random.default_rng(5)
        el, cs = (rq(rng), rq(rng)), rq(rng)
        air = {"poseidon": lambda: airs.PoseidonEval(log, el, cs), "plonk": lambda: airs.PlonkEval(log, el, cs),
               "wide_fib": lambda: airs.WideFibonacciEval(log, 100)}[name]()
        t_c = time.perf_counter()
        gc = codegen.GeneratedComponent(air)
        compile_s = time.perf_counter() - t_c
        N = 1 << air.max_constraint_log_degree_bound()
        n_cols = gc.n_cols
        block = torch.randint(0, P, (n_cols, N), dtype=torch.int64, device="cuda").to(torch.int32)
        ptrs = [block[i].data_ptr() for i in range(n_cols)]
        acc = [torch.zeros(N, dtype=torch.int32, device="cuda") for _ in range(4)]
        accp = [a.data_ptr() for a in acc]
        pw = (_lib.QM31 * gc.n_constraints)(*[_lib.QM31(rq(rng)) for _ in range(gc.n_constraints)])
        stream = torch.cuda.current_stream().cuda_stream

        def gen():
            gc.eval_constraints(ptrs, pw, accp, stream)

        def timed(fn):
            for _ in range(args.warmup):
                fn()
            barrier()
            ts = []
            for _ in range(args.steps):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record()
                fn()
                e1.record()
                e1.synchronize()
                ts.append(e0.elapsed_time(e1))
            return max_over_ranks(float(np.median(ts)))

        ms = timed(gen)
        algo = 4 * n_cols * N + 32 * N  # column words read, accumulation column read and written
        rec = {"rows": N, "columns": n_cols, "constraints": gc.n_constraints, "generated_ms": ms,
               "generated_gbs": algo / ms / 1e6, "generated_frac_hbm": algo / ms / 1e6 / peak,
               "nvrtc_compile_s": compile_s}
        if hand_id is not None:
            els = (_lib.QM31 * 2)(_lib.QM31(el[0]), _lib.QM31(el[1]))
            comp = _lib.Component(hand_id, log, 100 if hand_id == 0 else 0, _lib.QM31(cs),
                                  els if hand_id == 1 else None, 2 if hand_id == 1 else 0)
            tab = (C.c_void_p * n_cols)(*ptrs)
            a4 = (C.c_void_p * 4)(*accp)

            def hand():
                _lib.call("stwo_eval_constraints", C.byref(comp), tab, n_cols, pw, gc.n_constraints, a4, stream)

            hms = timed(hand)
            rec.update({"hand_written_ms": hms, "hand_written_gbs": algo / hms / 1e6})
        out[f"{name}_2e{log}"] = rec
        del block, acc
        torch.cuda.empty_cache()
    if rank != 0:
        return
    pos = out[f"poseidon_2e{specs[0][1]}"]
    line = {
        "metric": f"constraint evaluation rows/s (Poseidon2 2^{specs[0][1]} rows on the "
                  f"2^{specs[0][1] + 2}-point evaluation domain, generated kernel)",
        "value": pos["rows"] * world / (pos["generated_ms"] / 1e3), "unit": "rows/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": pos["generated_ms"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32 (M31 field words)",
        "data": "synthetic: uniform column words (seed 5)",
        "config": {"workload": "constraint point-wise eval: Poseidon2 2^16, Plonk 2^20, wide-Fibonacci 2^20 x 100",
                   "l2": "columns (1.36 GB for Poseidon2) larger than L2; no flush",
                   "parallelism": f"replicas x{world}"},
        "airs": out,
        "roofline": {"bound": "hbm", "kernel": "generated Poseidon2 constraint kernel",
                     "achieved": pos["generated_gbs"], "peak": peak, "unit": "GB/s",
                     "frac": pos["generated_frac_hbm"], "peak_kind": peak_kind, "traffic": None},
    }
    print(json.dumps(line), flush=True)


def run_gb300(args):
    import numpy as np
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from stwo_gb300 import _lib
    from stwo_gb300.build import build_backend

    if rank == 0 or world == 1:
        build_backend()
    if world > 1:
        torch.distributed.barrier()
    _lib.call("stwo_device_init", local)
    lib = _lib.load()

    from stwo_gb300 import replicas

    ranks = replicas.Ranks(world, rank, local)

    def barrier():
        replicas.barrier(ranks)

    def max_over_ranks(v):
        return replicas.max_over_ranks(v, ranks)

    if args.workload == "kernels":
        return run_kernels(args, world, rank, local, lib, barrier, max_over_ranks)
    if args.workload == "gkr":
        return run_gkr(args, world, rank, local, lib, barrier, max_over_ranks)
    if args.workload == "batch":
        return run_batch(args, world, rank, local, lib, barrier, max_over_ranks)
    if args.workload == "serve":
        return run_serve(args, world, rank, local, lib, barrier, max_over_ranks)
    if args.workload == "blake_round":
        return run_blake_round(args, world, rank, local, lib, barrier, max_over_ranks)
    if args.workload == "constraints":
        return run_constraints(args, world, rank, local, lib, barrier, max_over_ranks)
    if args.workload == "blake_full":
        return run_blake_full(args, world, rank, local, lib, barrier, max_over_ranks)

    wl = PoseidonWorkload(log=args.log_rows)
    for _ in range(args.warmup):
        wl.step()
    barrier()
    launches0 = lib.stwo_kernel_launches()
    times = []
    with ClockSampler(local) as clk:
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            wl.step()
            e1.record()
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        barrier()
        wall = time.perf_counter() - t0
    launches = lib.stwo_kernel_launches() - launches0
    step_ms = max_over_ranks(float(np.mean(times)))
    step_spread = {"min": float(np.min(times)), "median": float(np.median(times)), "max": float(np.max(times))}
    # End to end: initial states from pinned host memory, proof bytes back on the host.
    for _ in range(max(1, args.warmup // 2)):
        wl.step(from_host=True)
    barrier()
    et = []
    for _ in range(args.steps):
        t1 = time.perf_counter()
        wl.step(from_host=True)
        torch.cuda.synchronize()
        et.append((time.perf_counter() - t1) * 1e3)
    e2e_ms = max_over_ranks(float(np.mean(et)))
    # One extra proof with per-stage device timing (outside the timed region).
    _lib.call("stwo_set_stage_timing", 1)
    wl.step()
    names = (C.c_char_p * 64)()
    ms = (C.c_float * 64)()
    k = lib.stwo_stage_times(names, ms, 64)
    _lib.call("stwo_set_stage_timing", 0)
    stages = {names[i].decode(): float(ms[i]) for i in range(min(k, 64))}
    if rank != 0:
        return
    peak, peak_kind = measured_peaks()
    sbytes = wl.stage_bytes()
    hbm_stages = {k2: v for k2, v in stages.items() if k2 in sbytes and v > 0}
    dom = max(hbm_stages, key=hbm_stages.get) if hbm_stages else None
    roof = None
    if dom:
        ach = sbytes[dom] / (hbm_stages[dom] / 1e3) / 1e9
        roof = {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                "peak_kind": peak_kind, "traffic": wl.stage_traffic().get(dom),
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the stage's kernels at "
                                  "2^14 rows, scaled by the rows (2-pass FFT: intermediate written and re-read)",
                "algorithmic_bytes_per_launch": sbytes[dom],
                "stage_ms": hbm_stages[dom]}
        if dom == "Composition extension":
            # What actually bounds the stage: the butterfly's integer datapath. The composition
            # extension evaluates each column of 2^LOG coefficients on the 2^(LOG + 2)-point
            # domain, four sub-domains of LOG layers of 2^(LOG - 1) butterflies each.
            bfly = wl.TRACE_COLS * 4 * wl.LOG * (1 << (wl.LOG - 1))
            roof["int_bound"] = int_bound("butterfly", bfly / (hbm_stages[dom] / 1e3), clk.summary(), local)
            roof["int_bound"]["butterflies_per_launch"] = bfly
    line = {
        "metric": "proof s & trace cells/s (Poseidon2 2^16 rows)",
        "value": wl.cells * world / (step_ms / 1e3),
        "unit": "trace cells/s",
        "proof_s": step_ms / 1e3,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": step_ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u32 (M31 field words)",
        "data": "synthetic: seeded uniform M31 initial states (splitmix64 mod P)",
        "config": poseidon_config(wl.LOG, world),
        "proof_bytes": len(wl.proof),
        "ms_per_step_spread": step_spread,
        "stages_ms": stages,
        "roofline": roof,
        "e2e": {"value": wl.cells * world / (e2e_ms / 1e3), "unit": "trace cells/s", "proof_s": e2e_ms / 1e3,
                "h2d_bytes_per_step": wl.host_in.numel() * 4, "d2h_bytes_per_step": len(wl.proof),
                "input_path": "initial states in pinned host memory, read by the trace kernel over the host link"},
        "gpu_launches": int(launches),
        "wall_s": wall,
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline and world == 1:  # the CPU baseline is timed at N=1 only
        line["cpu_baseline"] = cpu_baseline_poseidon(args.cpu_threads, log=wl.LOG)
    if world == 1 and args.steps >= 3 and not args.log_rows:
        # The batched and served forms of the same prover, measured after (and outside) the timed
        # region of the headline proof with fewer steps, so that one default run records all three.
        side = argparse.Namespace(**{**vars(args), "steps": 5, "warmup": 2})
        b = run_batch(side, world, rank, local, lib, barrier, max_over_ranks, emit=False)
        line["batch"] = {k: b[k] for k in ("metric", "value", "unit", "ms_per_step", "plain", "speedup_vs_plain",
                                           "plain_breakdown", "proofs_identical_to_plain", "e2e", "gpu_launches",
                                           "clocks", "autotune")}
        side = argparse.Namespace(**{**vars(args), "steps": 3, "warmup": 1})
        v = run_serve(side, world, rank, local, lib, barrier, max_over_ranks, emit=False)
        line["serve"] = {k: v[k] for k in ("metric", "value", "unit", "p50_ms", "plain", "p99_vs_plain",
                                           "throughput_proofs_per_s", "proofs_identical_to_plain", "clocks")}
        line["side_measurements"] = ("batch (5 steps) and serve (3 rounds of 200 requests) run after the timed "
                                     "region; the headline value is the single proof")
    print(json.dumps(line), flush=True)


def poseidon_config(log, world):
    """The `config` of the Poseidon2 proof workload, shared by both arms."""
    cfg = PoseidonWorkload.CFG
    return {"workload": f"Poseidon2 AIR proof, 2^{log} rows x 8 permutations, LogUp interaction trace",
            "log_n_rows": log, "trace_cells": (1 << log) * PoseidonWorkload.TRACE_COLS, "pow_bits": cfg[0],
            "log_blowup": cfg[1], "log_last_layer": cfg[2], "n_queries": cfg[3],
            "l2": "working set (~3 GB at 2^16 rows) far larger than L2; no flush",
            "parallelism": f"replicas x{world}"}


def cpu_baseline_poseidon(threads=0, log=16):
    """The oracle's Poseidon2 proof on all host cores (OpenMP), a bounded sample of 2^log rows."""
    import oracle.pyoracle as O

    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    nthreads = threads or os.cpu_count() or 1
    init = gen_words(3, 0, (1 << log) * 8 * 16)
    t0 = time.perf_counter()
    O.prove_poseidon(log, init, PoseidonWorkload.CFG)
    secs = time.perf_counter() - t0
    cells = (1 << log) * PoseidonWorkload.TRACE_COLS
    return {"value": cells / secs, "unit": "trace cells/s", "cores": nthreads, "kind": "port",
            "proof_s": secs, "sample": f"one whole Poseidon2 proof of 2^{log} rows, the benchmarked "
                                        f"configuration itself (same AIR, PcsConfig and input generator): "
                                        f"{secs:.2f} s"}


def run_kernels(args, world, rank, local, lib, barrier, max_over_ranks):
    import numpy as np
    import torch

    wl = KernelsWorkload(n_cols=args.n_cols)

    # Warm-up.
    for _ in range(args.warmup):
        wl.restore()
        wl.stages()
    barrier()

    # Timed: device-resident inputs; per-stage CUDA events on the launching stream.
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(6)] for _ in range(args.steps)]
    launches0 = lib.stwo_kernel_launches()
    with ClockSampler(local) as clk:
        barrier()
        t0 = time.perf_counter()
        for s in range(args.steps):
            wl.restore()
            wl.stages(evs[s])
        barrier()
        wall = time.perf_counter() - t0
    launches = lib.stwo_kernel_launches() - launches0
    stage_ms = np.zeros(5)
    for s in range(args.steps):
        for i in range(5):
            stage_ms[i] += evs[s][i].elapsed_time(evs[s][i + 1])
    stage_ms /= args.steps
    step_ms = max_over_ranks(float(stage_ms.sum()))

    # End to end through the public API: pinned host inputs -> HBM -> hot path -> root + FRI layer.
    for _ in range(max(1, args.warmup)):
        wl.work.copy_(wl.host_in, non_blocking=True)
        wl.stages()
        wl.readback()
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        wl.work.copy_(wl.host_in, non_blocking=True)
        wl.stages()
        wl.readback()
    e1.record()
    barrier()
    e2e_ms = max_over_ranks(e0.elapsed_time(e1) / args.steps)

    if rank != 0:
        return
    peak, peak_kind = measured_peaks()
    N, n = 1 << wl.L, 1 << wl.LOG
    # Dominant HBM-bound kernel: the evaluate pass (4n read + 4N written per column).
    eval_bytes = wl.N_COLS * (4 * n + 4 * N)
    eval_s = stage_ms[1] / 1e3
    achieved = eval_bytes / eval_s / 1e9
    interp_gbs = wl.N_COLS * 8 * n / (stage_ms[0] / 1e3) / 1e9
    comp = N * ((wl.N_COLS + 15) // 16)  # leaf compressions = N * ceil(columns / 16)
    line = {
        "metric": "trace cells/s (kernel microbench: interpolate+evaluate 256x2^20 @ blowup 4, "
                  "Blake2s Merkle 256x2^22, FRI fold 2^22->2^4)",
        "value": wl.cells * world / (step_ms / 1e3),
        "unit": "cells/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": step_ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u32 (M31 field words)",
        "data": "synthetic seeded (splitmix64 mod P), shapes of the kernel microbench config",
        "config": {"workload": "kernels: 256 cols x 2^20 -> 2^22 (blowup 4) + Merkle + FRI 2^22->2^4",
                   "n_cols": wl.N_COLS, "log_size": wl.LOG, "log_blowup": wl.BLOWUP, "fri_log": wl.FRI_LOG,
                   "l2": "inputs (1 GiB) larger than L2; no flush", "parallelism": f"replicas x{world}"},
        "stages_ms": {"interpolate": stage_ms[0], "evaluate": stage_ms[1], "merkle_leaves": stage_ms[2],
                      "merkle_nodes": stage_ms[3], "fri_folds": stage_ms[4]},
        "roofline": {"bound": "hbm", "kernel": "evaluate 2^20 -> 2^22: k_fft_reg + k_fft_tile passes (integer-bound: see int_bound)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": None,
                     "algorithmic_bytes_per_call": eval_bytes},
        "interpolate_gbs": interp_gbs,
        "merkle_leaf_compressions_per_s": comp / (stage_ms[2] / 1e3),
        # Both stages are bound by the integer datapath, not HBM: each against the library's
        # register-only probe of its inner operation. The evaluation runs 2^b sub-domain FFTs of
        # LOG layers of 2^(LOG-1) butterflies per column.
        "int_bound": {
            "evaluate": int_bound("butterfly", wl.N_COLS * (1 << wl.BLOWUP) * wl.LOG * (1 << (wl.LOG - 1))
                                  / (stage_ms[1] / 1e3), clk.summary(), local),
            "merkle_leaves": int_bound("blake2s", comp / (stage_ms[2] / 1e3), clk.summary(), local)},
        "e2e": {"value": wl.cells * world / (e2e_ms / 1e3), "unit": "cells/s",
                "h2d_bytes_per_step": wl.cells * 4, "d2h_bytes_per_step": 32 + 4 * 4 * (1 << wl.FRI_LAST),
                "ms_per_step": e2e_ms},
        "gpu_launches": int(launches // args.steps) * args.steps,
        "wall_s": wall,
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline and world == 1:  # the CPU baseline is timed at N=1 only
        line["cpu_baseline"] = cpu_baseline_kernels(args.cpu_threads)
    print(json.dumps(line), flush=True)


def cpu_baseline_kernels(threads=0, n_cols=16):
    """The oracle on all host cores over a bounded sample (n_cols columns at full sizes)."""
    import numpy as np

    import oracle.pyoracle as O

    lib = O.lib()
    lib.oracle_bench_cfg2.restype = C.c_double
    root = np.zeros(8, np.uint32)
    fri = np.zeros(64, np.uint32)
    nthreads = threads or os.cpu_count() or 1
    secs = lib.oracle_bench_cfg2(C.c_uint32(n_cols), C.c_uint32(20), C.c_uint32(2), C.c_uint32(22),
                                 C.c_int(nthreads), root.ctypes.data_as(C.c_void_p), fri.ctypes.data_as(C.c_void_p))
    return {"value": n_cols * (1 << 20) / secs, "unit": "cells/s", "cores": nthreads, "kind": "port",
            "sample": f"{n_cols} of 256 columns at full sizes (2^20 -> 2^22, Merkle over {n_cols} cols, "
                      f"FRI 2^22->2^4): {secs:.2f} s"}


def run_reference(args):
    """The reference arm: the oracle (C++ restatement of the reference CPU prover; the Rust crate
    needs cargo, which this image lacks) on all host cores. Rank 0 only."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from stwo_gb300.build import build_oracle

    build_oracle()
    if args.workload == "kernels":
        for _ in range(args.warmup):
            cpu_baseline_kernels(args.cpu_threads, n_cols=4)
        vals = [cpu_baseline_kernels(args.cpu_threads, n_cols=8) for _ in range(args.steps)]
        metric = ("trace cells/s (kernel microbench: interpolate+evaluate 256x2^20 @ blowup 4, "
                  "Blake2s Merkle 256x2^22, FRI fold 2^22->2^4)")
        unit = "cells/s"
        config = {"workload": "kernels: 256 cols x 2^20 -> 2^22 (blowup 4) + Merkle + FRI 2^22->2^4",
                  "sample_cols_per_step": 8}
    elif args.workload == "gkr":
        for _ in range(min(args.warmup, 1)):
            cpu_baseline_gkr(args.cpu_threads)
        vals = [cpu_baseline_gkr(args.cpu_threads) for _ in range(args.steps)]
        metric = "GKR prove_batch leaves/s (LogUp generic, 2^20 leaves)"
        unit = "leaves/s"
        config = {"workload": "GKR batch proof, one LogUp-generic layer of 2^20 leaves (Poseidon2 relation shape "
                              "at 2^16 rows)", "log_leaves": 20}
    elif args.workload == "blake_full":
        import oracle.pyoracle as O

        log = args.log_rows or 10

        def one():
            t0 = time.perf_counter()
            O.prove_blake(log, (5, 1, 0, 3))
            dt = time.perf_counter() - t0
            return {"value": (1 << log) / dt, "unit": "BLAKE2s instances/s", "proof_s": dt,
                    "cores": os.cpu_count(), "kind": "port",
                    "sample": f"one whole prove_blake of 2^{log} instances"}

        for _ in range(min(args.warmup, 1)):
            one()
        vals = [one() for _ in range(args.steps)]
        metric = f"full Blake example proof s & BLAKE2s instances/s (2^{log} instances)"
        unit = "BLAKE2s instances/s"
        config = {"workload": f"prove_blake, 2^{log} instances", "log_instances": log, "pcs_config": [5, 1, 0, 3]}
    else:
        # Each step is one whole proof of the benchmarked configuration (2^16 rows: ~2-3 s on 16
        # cores), so both arms time the same work.
        log = args.log_rows or PoseidonWorkload.LOG
        for _ in range(min(args.warmup, 1)):
            cpu_baseline_poseidon(args.cpu_threads, log=log)
        vals = [cpu_baseline_poseidon(args.cpu_threads, log=log) for _ in range(args.steps)]
        metric = "proof s & trace cells/s (Poseidon2 2^16 rows)"
        unit = "trace cells/s"
        config = poseidon_config(log, int(os.environ.get("WORLD_SIZE", "1")))
    v = sorted(x["value"] for x in vals)[len(vals) // 2]
    cb = dict(vals[0])
    cb["value"] = v
    out = {
        "impl": "reference", "metric": metric, "value": v, "unit": unit,
        "n_gpus": int(os.environ.get("WORLD_SIZE", "1")), "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": float(sorted(x.get("proof_s", 0) for x in vals)[len(vals) // 2]) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32 (M31 field words)",
        "data": "synthetic seeded (splitmix64 mod P)", "config": config, "cpu_baseline": cb,
        "e2e": {"value": v, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "C++ restatement of the reference CPU prover (the Rust reference needs cargo, absent here)",
    }
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="poseidon", choices=["poseidon", "kernels", "gkr", "batch", "serve",
                                                                "blake_round", "constraints", "blake_full"],
                    help="poseidon: the headline Poseidon2 2^16-row proof; kernels: the kernel microbench; "
                         "gkr: GKR batch proof of 2^20 LogUp leaves; batch: 64 mixed proofs on a worker pool; "
                         "serve: Poisson-arrival serving with latency percentiles; blake_round: one proof of the "
                         "Blake2s round AIR; constraints: generated vs hand-written constraint kernels; "
                         "blake_full: one proof of the full Blake example (framework path)")
    ap.add_argument("--workers", type=int, default=0, help="worker streams of the batch (16) / serve (8) workloads")
    ap.add_argument("--requests", type=int, default=0, help="requests of the serve workload (200)")
    ap.add_argument("--cpu-threads", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--n-cols", type=int, default=0, help="columns of the kernel workload (default 256; "
                    "smaller only for profiling captures)")
    ap.add_argument("--log-rows", type=int, default=0, help="log2 rows of the Poseidon2 workload (default 16; "
                    "smaller only for profiling captures)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
