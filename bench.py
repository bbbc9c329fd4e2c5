"""Benchmark of the GB300 RNS-BFV hot path.

Workload (one step): `Multiplicator::multiply` with relinearization on a batch
of 64 ciphertext pairs at N = 2^14 with six 62-bit moduli, the default
extension basis of seven 62-bit primes, t = 65537, relinearization key
resident on the device, the pipeline recorded once as a CUDA graph and
replayed. Ciphertexts are synthetic: real encryptions made by the CPU oracle
from a seeded RNG. The metric is ciphertext products per second (whole job).
Besides the device-resident number the line carries:
  direct_calls  the same batch without the graph;
  e2e           the same metric through the host entry point (pinned host
                buffers, H2D + compute + D2H inside the timed region);
  single        64 one-ciphertext launches (the unbatched GPU path);
  roofline      the batched NTT kernels against the measured HBM bandwidth;
  cpu_baseline  the oracle (C++/Python restatement of fhe.rs) on host cores.
`--impl reference` times the CPU restatement alone on all host cores.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N, L, T = 1 << 14, 6, 65537
METRIC = "BFV mul+relin ct/s N=2^14 L=6, batched vs single, bit-exact; NTT % HBM peak"
UNIT = "ct/s"
# Algorithmic traffic of each stage of one product, in limbs of 8N bytes
# (L = 6 ciphertext moduli, M = 13 extended, Lk = 6 key moduli): what a stage
# must read and write at least once; twiddle tables stay in L2.
STAGE_LIMBS = {
    "A": 8 * L,                      # read + write the 4 operands
    "B": 4 * L + 4 * (2 * L + 1 - L),  # read 4L, write 4(M - L)
    "C": 8 * (2 * L + 1 - L),        # read + write the extension limbs
    "D": 4 * (2 * L + 1) + 3 * (2 * L + 1),  # read 4M operand limbs, write 3M
    "E": 3 * (2 * L + 1) + 2 * L + L * L,  # read 3M; write c0, c1 and the L * Lk digit rows
    "F": 2 * (L * L + 2 * L),        # read + write the digit rows and c0, c1 (block passes)
    "G": L * L + 4 * L,              # read the digit NTTs, read + write c0, c1 (keys added per batch)
}
STAGE_KERNELS = {
    "A": "k_ntt_inv<12, SrcPair> (inverse NTT of the operands, block pass; its strided last stages run in B)",
    "B": "k_rns_scale<6, 8> (A's strided last stages, extension 6 -> 7 new moduli, C's strided first stages)",
    "C": "k_ntt_fwd<12> (forward NTT of the extension limbs, block pass)",
    "D": "k_ntt_inv<12, SrcTensor> (tensor product + inverse NTT, block pass; its strided last stages run in E)",
    "E": "k_rns_scale<13, 8> (D's strided last stages, t/Q scale-down 13 -> 6, F's strided first stages and "
         "digit expansion)",
    "F": "k_ntt_fwd<12>, twice (digit NTTs in every key modulus, then c0/c1 NTTs; block passes)",
    "G": "k_key_mac (key inner product)",
}
# Kernel launches of each stage under the same plan.
STAGE_LAUNCHES = {"A": 1, "B": 1, "C": 1, "D": 1, "E": 1, "F": 2, "G": 1}
# DRAM bytes (read + write) of each stage's kernels for one 64-pair
# multiplication with the plan A,C,D,F = 12 (2^12-residue blocks; every
# strided NTT stage applied inside the RNS scalers B and E; E's sums on the
# tensor cores), from the ncu capture summarised in
# profiles/stages_mul_relin_n16384_b64.md.
STAGE_TRAFFIC_BYTES = {"A": 353.2e6, "B": 393.2e6, "C": 409.4e6, "D": 728.0e6, "E": 675.7e6, "F": 696.2e6,
                       "G": 493.6e6}
# The ncu figures above and below hold for the library sources they were
# captured on: library_source_hash() of that tree. A run on other sources
# reports null for them instead of stale numbers.
PROFILED_SOURCE_HASH = "e7052cef359c4eb3"
# Share of the elapsed cycles in which the integer multipliers (the FMA-heavy
# pipe, which executes every IMAD) were busy, per stage, from the same ncu
# capture of one 64-pair multiplication (F: time-weighted over its two
# launches); the whole multiplication, time-weighted.
STAGE_FMAHEAVY_PCT = {"A": 69.9, "B": 84.0, "C": 70.6, "D": 67.1, "E": 61.3, "F": 70.4, "G": 63.7}
MULTIPLY_FMAHEAVY_PCT = 69.3


def library_source_hash() -> str:
    """SHA-256 (first 16 hex digits) of the library's sources: every file of
    fhe.rs_gb300/csrc and include/, in name order."""
    import hashlib

    h = hashlib.sha256()
    for d in (os.path.join(ROOT, "fhe.rs_gb300", "csrc"), os.path.join(ROOT, "include")):
        for name in sorted(os.listdir(d)):
            with open(os.path.join(d, name), "rb") as f:
                h.update(name.encode() + b"\0" + f.read())
    return h.hexdigest()[:16]


def cpu_model() -> str:
    """The host CPU's model name (or architecture when none is listed)."""
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                key = line.split(":")[0].strip().lower()
                if key in ("model name", "cpu model", "hardware"):
                    return line.split(":", 1)[1].strip()
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform

    return platform.machine()


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []
        self.first = 0  # index of the first sample taken once the region started
        self._got = threading.Event()

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
            # nvidia-smi takes a few hundred ms to start: wait (bounded) for
            # its first sample so that short timed regions are covered.
            self._got.wait(timeout=3.0)
            self.first = len(self.lines)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())
            self._got.set()

    def __exit__(self, *a):
        if self.proc is not None:
            # A region shorter than the sampling period still gets the sample
            # that follows it (at most one period later).
            deadline = time.time() + 0.5
            while len(self.lines) <= self.first and time.time() < deadline and self.proc.poll() is None:
                time.sleep(0.01)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        for ln in self.lines[self.first:] or self.lines[-1:]:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no nvidia-smi sample"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def make_inputs(ora, batch: int, seed: int = 2026, distinct: int = 16, degree: int = N, moduli: int = L):
    """Keys and `batch` ciphertext pairs (cycled from `distinct` encryptions)."""
    rng = np.random.default_rng(seed)
    par = ora.BfvParameters(degree, T, moduli_sizes=[62] * moduli)
    sk = ora.SecretKey.random(par, rng)
    rk = ora.RelinearizationKey(sk, rng)
    cts = [sk.encrypt(ora.Plaintext.encode(rng.integers(0, T, degree, dtype=np.uint64), "simd", par), rng)
           for _ in range(distinct)]
    arrs = [c.to_array() for c in cts]
    lhs = np.stack([arrs[i % distinct] for i in range(batch)])
    rhs = np.stack([arrs[(7 * i + 3) % distinct] for i in range(batch)])
    return par, sk, rk, cts, lhs, rhs


def measure_mixed_levels(fg, ora, torch, par_o, sk, per_level: int = 16, reps: int = 20):
    """A 64-pair batch spread over levels 0-3 (16 pairs each, the level-2
    group relinearized by a key at level 0, which switches down after the key
    switch), issued as one multiply_groups call: one multiplicator per level,
    the groups overlapping on side streams. The first product of every group
    is checked against the oracle before timing."""
    rng = np.random.default_rng(77)
    par = fg.BfvParameters(N, par_o.moduli, T)
    mults, lhs, rhs, first = [], [], [], []
    for lvl, klvl in [(0, 0), (1, 1), (2, 0), (3, 3)]:
        rk_o = ora.RelinearizationKey(sk, rng, lvl, klvl)
        rk = fg.RelinearizationKey(par, rk_o.ksk.c0_array(), rk_o.ksk.c1_array(), lvl, klvl)
        mults.append(fg.Multiplicator.default(rk))
        cts = [sk.encrypt(ora.Plaintext.encode(rng.integers(0, T, N, dtype=np.uint64), "simd", par_o, lvl), rng)
               for _ in range(4)]
        arrs = [c.to_array() for c in cts]
        lhs.append(fg.to_device(np.stack([arrs[i % 4] for i in range(per_level)])))
        rhs.append(fg.to_device(np.stack([arrs[(i + 1) % 4] for i in range(per_level)])))
        first.append((ora.Multiplicator.default(rk_o), cts[0], cts[1]))
    outs = fg.multiply_groups(mults, lhs, rhs)
    torch.cuda.synchronize()
    for g, (mo, a, b) in enumerate(first):
        if not np.array_equal(fg.to_host(outs[g][:1])[0], mo.multiply(a, b).to_array()):
            raise SystemExit(f"bench: mixed-level group {g} is not bit-exact with the oracle")
    for _ in range(3):
        fg.multiply_groups(mults, lhs, rhs, outs)
    stream = torch.cuda.current_stream()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    start.record(stream)
    for _ in range(reps):
        fg.multiply_groups(mults, lhs, rhs, outs)
    end.record(stream)
    torch.cuda.synchronize()
    ms = start.elapsed_time(end) / reps
    return {"value": 4 * per_level / (ms / 1000.0), "unit": UNIT, "ms_per_step": ms,
            "note": f"{4 * per_level} pairs at levels 0-3 ({per_level} each; level 2 with its key at level 0) "
                    "in one multiply_groups call"}


def max_over_ranks(ms: float, dist) -> float:
    """The slowest rank's step time (replicas: every rank runs its own batch)."""
    import torch

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([ms], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(batch: int, ms: float, world: int) -> float:
    """Whole-job products per second: every rank multiplies `batch` pairs per
    step of `ms` milliseconds (the slowest rank's)."""
    return world * batch / (ms / 1000.0)


def cpu_multiply_rate(driver, cts, threads: int, per_thread: int):
    """Products per second of the CPU restatement of Multiplicator::multiply
    (oracle.cpp's whole-product loop, no Python inside) on `threads` host
    threads, `per_thread` independent pairs each (the reference has no
    internal parallelism; callers parallelise over ciphertexts)."""
    count = threads * per_thread
    arrs = [c.to_array() for c in cts]
    lhs = np.stack([arrs[k % len(arrs)] for k in range(count)])
    rhs = np.stack([arrs[(3 * k + 1) % len(arrs)] for k in range(count)])
    t0 = time.perf_counter()
    driver.multiply(lhs, rhs, threads)
    dt = time.perf_counter() - t0
    return count / dt, dt


def cpu_baseline_sample(ora, rk, cts, seconds: float):
    """Single-thread and all-core rates of the CPU restatement, the all-core
    sample sized to about `seconds` of wall time."""
    driver = ora.MultiplyDriver(ora.Multiplicator.default(rk))
    cores = os.cpu_count() or 1
    cpu_multiply_rate(driver, cts, 1, 1)  # warm the caches
    single, _ = cpu_multiply_rate(driver, cts, 1, 3)
    rate0, _ = cpu_multiply_rate(driver, cts, cores, 1)
    per_thread = max(1, int(seconds * rate0 / cores))
    rate, dt = cpu_multiply_rate(driver, cts, cores, per_thread)
    return {"value": rate, "unit": UNIT, "cores": cores, "kind": "port", "single_thread": single,
            "cpu": cpu_model(),
            "sample": f"{cores * per_thread} products on {cores} host threads ({dt:.1f} s), single-thread "
                      f"{single:.2f} ct/s; C++ restatement of fhe.rs Multiplicator::multiply "
                      "(oracle.cpp, -O3 -mcpu/-march=native, std::thread over independent pairs); the Rust "
                      "reference cannot be built here"}


def run_reference(args, rank: int):
    from oracle import build as oracle_build
    from oracle import ora

    if rank != 0:
        return
    oracle_build.build()
    par, sk, rk, cts, _, _ = make_inputs(ora, 8, distinct=8)
    driver = ora.MultiplyDriver(ora.Multiplicator.default(rk))
    cores = os.cpu_count() or 1
    # One step = the GPU arm's batch of products, spread over every host core.
    per_thread = -(-args.batch // cores)
    cpu_multiply_rate(driver, cts, 1, 1)  # warm the caches of the oracle
    for _ in range(max(args.warmup, 0)):
        cpu_multiply_rate(driver, cts, cores, per_thread)
    total = 0.0
    for _ in range(args.steps):
        total += cpu_multiply_rate(driver, cts, cores, per_thread)[1]
    value = args.steps * cores * per_thread / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": {"workload": "bfv_mul_relin_batched", "degree": N, "moduli": L, "moduli_bits": 62,
                   "extension_moduli": 7, "plaintext": T, "batch_pairs": cores * per_thread,
                   "keys": "resident in host memory", "parallelism": f"{cores} host threads"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "cpu": cpu_model(),
                         "sample": f"{cores * per_thread} products per step ({per_thread} per host thread) of the "
                                   "C++ restatement of fhe.rs Multiplicator::default().multiply (oracle.cpp, "
                                   "std::thread over independent pairs); the Rust reference cannot be built "
                                   "(no Rust toolchain)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, rank: int, world: int):
    import torch

    import __graft_entry__ as ge
    from oracle import ora

    ge.build()
    fg = ge.load_package()
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    B = args.batch
    par_o, sk, rk_o, cts, lhs, rhs = make_inputs(ora, B)
    par = fg.BfvParameters(N, par_o.moduli, T)
    rk = fg.RelinearizationKey(par, rk_o.ksk.c0_array(), rk_o.ksk.c1_array())
    mult = fg.Multiplicator.default(rk)
    fg.rns_tensor_set(args.rns_tensor == "on")
    lhs_d, rhs_d = fg.to_device(lhs), fg.to_device(rhs)
    out_d = fg.empty((B, 2, L, N))
    stream = torch.cuda.current_stream()
    logn = N.bit_length() - 1
    if args.ntt_block == "auto":
        mult.autotune(B)
    else:
        fg.ntt_plan_set(logn, int(args.ntt_block))
    ntt_block = dict(zip(["A", "C", "D", "F", "F_split", "D_split"], mult.plan))

    # Parity gate: two products of the batch against the oracle.
    mult.multiply(lhs_d, rhs_d, out_d)
    torch.cuda.synchronize()
    got = fg.to_host(out_d)
    mult_o = ora.Multiplicator.default(rk_o)
    for b in (0, B - 1):
        lo = ora.Ciphertext.from_array(par_o, lhs[b], 0)
        ro = ora.Ciphertext.from_array(par_o, rhs[b], 0)
        if not np.array_equal(got[b], mult_o.multiply(lo, ro).to_array()):
            raise SystemExit(f"bench: GPU product {b} is not bit-exact with the oracle")

    # The step: the whole batched pipeline recorded once as a CUDA graph and
    # replayed (the graph reads lhs_d / rhs_d and writes out_d at replay).
    graph = mult.capture(lhs_d, rhs_d, out_d)
    for _ in range(args.warmup):
        graph.launch()
        mult.multiply(lhs_d, rhs_d, out_d)
    torch.cuda.synchronize()
    if not np.array_equal(fg.to_host(out_d), got):
        raise SystemExit("bench: graph replay differs from the direct call")
    if dist:
        dist.barrier()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = fg.kernel_launch_count()
    with ClockSampler(dev) as clocks:
        torch.cuda.synchronize()
        start.record(stream)
        for _ in range(args.steps):
            graph.launch()
        end.record(stream)
        torch.cuda.synchronize()
    launches = fg.kernel_launch_count() - launches0
    ms = start.elapsed_time(end) / args.steps
    # The same batch through direct calls (one launch call per kernel).
    start.record(stream)
    for _ in range(args.steps):
        mult.multiply(lhs_d, rhs_d, out_d)
    end.record(stream)
    torch.cuda.synchronize()
    direct_ms = start.elapsed_time(end) / args.steps
    if dist:
        ms = max_over_ranks(ms, dist)
        dist.barrier()
    value = replica_throughput(B, ms, world)

    # The unbatched path: 64 one-ciphertext launches.
    one_l, one_r, one_o = lhs_d[:1], rhs_d[:1], out_d[:1]
    for _ in range(3):
        mult.multiply(one_l, one_r, one_o)
    torch.cuda.synchronize()
    start.record(stream)
    for b in range(B):
        mult.multiply(lhs_d[b:b + 1], rhs_d[b:b + 1], out_d[b:b + 1])
    end.record(stream)
    torch.cuda.synchronize()
    single_ms = start.elapsed_time(end)
    single_rate = B / (single_ms / 1000.0)

    # End to end through the host entry point (pinned buffers).
    h_l = torch.from_numpy(lhs.view(np.int64)).pin_memory().numpy().view(np.uint64)
    h_r = torch.from_numpy(rhs.view(np.int64)).pin_memory().numpy().view(np.uint64)
    h_o = torch.empty((B, 2, L, N), dtype=torch.int64, pin_memory=True).numpy().view(np.uint64)
    for _ in range(2):
        mult.multiply_host(h_l, h_r, h_o)
    e2e_steps = max(3, args.steps // 2)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        mult.multiply_host(h_l, h_r, h_o)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    if not np.array_equal(h_o, got):
        raise SystemExit("bench: host entry point result differs from the device result")

    # Roofline of the batched NTT kernels: 256 polynomials x 6 limbs (201 MB,
    # larger than L2), forward and inverse timed separately.
    ctx = par.context_at_level(0)
    polys = 256
    buf = fg.to_device(np.tile(lhs[:1, 0], (polys, 1, 1)))
    fg.ntt_forward(ctx, buf)
    fg.ntt_backward(ctx, buf)
    torch.cuda.synchronize()
    reps = 10
    start.record(stream)
    for _ in range(reps):
        fg.ntt_forward(ctx, buf)
    end.record(stream)
    torch.cuda.synchronize()
    fwd_ms = start.elapsed_time(end) / reps
    start.record(stream)
    for _ in range(reps):
        fg.ntt_backward(ctx, buf)
    end.record(stream)
    torch.cuda.synchronize()
    inv_ms = start.elapsed_time(end) / reps
    data_bytes = 2 * 8 * polys * L * N  # read + write of every residue
    tw_bytes = 2 * 8 * L * N  # twiddles and their Shoup companions, one direction
    fwd_gbs = (data_bytes + tw_bytes) / (fwd_ms / 1000.0) / 1e9
    inv_gbs = (data_bytes + tw_bytes) / (inv_ms / 1000.0) / 1e9
    peak, peak_kind = _peaks()

    # Stage durations of the batched pipeline (events between stages, the
    # median of 5 runs) and the dominant stage's roofline.
    runs = [mult.stage_times(lhs_d, rhs_d, out_d) for _ in range(6)][1:]
    stage_ms = {k: statistics.median(r[k] for r in runs) for k in runs[0]}
    limb = 8 * N
    stage_bytes = {k: B * v * limb for k, v in STAGE_LIMBS.items()}
    stage_bytes["G"] += 2 * L * L * limb  # the relinearization key, read once per batch
    # The dominant kernel: the stage with the longest launch (per launch, as
    # stages C and F hold several kernels under the 2^12-block plan).
    dom = max(stage_ms, key=lambda k: stage_ms[k] / STAGE_LAUNCHES[k])
    dom_gbs = stage_bytes[dom] / (stage_ms[dom] / 1000.0) / 1e9

    # The NTT's butterflies per second against the measured butterfly
    # ceiling of this GPU (fheg_intpeak, register-resident Harvey
    # butterflies), and what 60% of the HBM bandwidth would need.
    probes, _ = measure_intpeak(fg, torch, kinds=(4, 5), steps=3)
    bfly = polys * L * butterflies_per_transform(logn)
    need_60 = 0.6 * peak * 1e9 / (data_bytes + tw_bytes) * bfly

    mixed = measure_mixed_levels(fg, ora, torch, par_o, sk)
    # The uneven-level rotation batch (N = 2^15, 32 ciphertexts at 4 to 12
    # moduli), after the headline's timed region.
    rotations = measure_rotations(fg, ora, torch, 32, 20, 3)
    # The batched NTT at the other degrees (256 polynomials x 6 limbs).
    ntt_degrees = measure_ntt_degrees(fg, ora, torch)

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline_sample(ora, rk_o, cts, args.cpu_seconds)

    # The ncu figures hold for one plan (A, C, D, F in 2^12 blocks) and one
    # source tree; any other run reports null for them.
    # (A plan entry of 0 means the process-wide plan of the degree.)
    src_hash = library_source_hash()
    traffic_plan_matches = all((ntt_block[k] or fg.ntt_plan_get(logn)) == 12 for k in ("A", "C", "D", "F")) \
        and src_hash == PROFILED_SOURCE_HASH
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded encryptions by the CPU oracle)",
            "config": {"workload": "bfv_mul_relin_batched", "degree": N, "moduli": L, "moduli_bits": 62,
                       "extension_moduli": 7, "plaintext": T, "batch_pairs": B, "keys": "device resident",
                       "ntt_block_logn": ntt_block, "rns_scaling": "tensor cores (tcgen05 byte-sliced products)"
                       if args.rns_tensor == "on" else "CUDA cores",
                       "step": f"one CUDA graph of {graph.kernels} kernels"
                       + (f" (two concurrent branches of {B // 2} and {B - B // 2} pairs)" if B >= 32 else ""),
                       "l2": "no flush: each step streams > 1 GB (inputs 201 MB, outputs 100 MB, scratch) through "
                             "the 126 MB L2", "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
            "single": {"value": single_rate, "unit": UNIT, "note": f"{B} one-ciphertext launches"},
            "direct_calls": {"value": B / (direct_ms / 1000.0), "unit": UNIT, "ms_per_step": direct_ms,
                             "note": "the batch without the graph"},
            "batch_vs_single": value / world / single_rate,
            "mixed_levels": mixed,
            "rotations": rotations,
            "ntt_degrees": ntt_degrees,
            "e2e": {"value": B / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(lhs.nbytes + rhs.nbytes),
                    "d2h_bytes_per_step": int(h_o.nbytes)},
            "roofline": {"bound": "hbm", "achieved": dom_gbs, "peak": peak, "unit": "GB/s", "frac": dom_gbs / peak,
                         "traffic": STAGE_TRAFFIC_BYTES.get(dom) if traffic_plan_matches else None,
                         "traffic_plan": "A,C,D,F = 2^12 blocks", "kernel": STAGE_KERNELS[dom],
                         "source_hash": src_hash, "profiled_source_hash": PROFILED_SOURCE_HASH,
                         "algorithmic_bytes": stage_bytes[dom], "launch_ms": stage_ms[dom], "peak_kind": peak_kind,
                         "note": "integer-multiplier bound, not HBM: all arithmetic is exact 64-bit residue "
                                 "arithmetic on the CUDA cores' 32-bit multipliers",
                         "int_pipe": {"kernel_fmaheavy_pct": STAGE_FMAHEAVY_PCT[dom] if traffic_plan_matches else None,
                                      "multiply_fmaheavy_pct": MULTIPLY_FMAHEAVY_PCT if traffic_plan_matches else None,
                                      "metric": "sm__pipe_fmaheavy_cycles_active.avg.pct_of_peak_sustained_elapsed",
                                      "source": "ncu, profiles/stages_mul_relin_n16384_b64.md"}},
            "stages": {k: {"ms": stage_ms[k], "gbs": stage_bytes[k] / (stage_ms[k] / 1000.0) / 1e9,
                           "kernel": STAGE_KERNELS[k]} for k in stage_ms},
            "ntt": {"kernel": "forward / inverse NTT alone, 256 polys x 6 limbs", "fwd_gbs": fwd_gbs,
                    "inv_gbs": inv_gbs, "fwd_frac": fwd_gbs / peak, "inv_frac": inv_gbs / peak, "fwd_ms": fwd_ms,
                    "inv_ms": inv_ms, "cluster": fg.ntt_cluster_get(logn),
                    "fwd_butterflies_per_s": bfly / (fwd_ms / 1000.0), "inv_butterflies_per_s": bfly / (inv_ms / 1000.0),
                    "fwd_butterfly_ceiling_per_s": probes[4]["ops_per_s"],
                    "inv_butterfly_ceiling_per_s": probes[5]["ops_per_s"],
                    "fwd_frac_of_ceiling": bfly / (fwd_ms / 1000.0) / probes[4]["ops_per_s"],
                    "inv_frac_of_ceiling": bfly / (inv_ms / 1000.0) / probes[5]["ops_per_s"],
                    "butterflies_per_s_for_60pct_hbm": need_60,
                    "note": "the butterfly ceiling is fheg_intpeak's register-resident Harvey butterfly: an NTT "
                            "at 60% of HBM needs more butterflies per second than the integer pipes issue"},
            "gpu_launches": int(launches),
            "clocks": clocks.summary(),
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def run_stages(args):
    """Stage breakdown of the batched multiplication (64 pairs at N = 2^14,
    L = 6 by default; --logn and --moduli choose another parameter set): W
    warm-up multiplies, then one multiply with events at the stage
    boundaries. Small enough to run under a profiler (14 launches a multiply)."""
    import torch

    import __graft_entry__ as ge
    from oracle import ora

    ge.build()
    fg = ge.load_package()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    B, n, nmod = args.batch, 1 << args.logn, args.moduli
    par_o, sk, rk_o, cts, lhs, rhs = make_inputs(ora, B, distinct=min(16, B), degree=n, moduli=nmod)
    par = fg.BfvParameters(n, par_o.moduli, T)
    rk = fg.RelinearizationKey(par, rk_o.ksk.c0_array(), rk_o.ksk.c1_array())
    mult = fg.Multiplicator.default(rk)
    if args.stage_plan:
        mult.plan = [int(x) for x in args.stage_plan.split(",")]
    lhs_d, rhs_d = fg.to_device(lhs), fg.to_device(rhs)
    out_d = fg.empty((B, 2, nmod, n))
    fg.rns_tensor_set(args.rns_tensor == "on")
    for _ in range(args.warmup):
        mult.multiply(lhs_d, rhs_d, out_d)
    runs = [mult.stage_times(lhs_d, rhs_d, out_d) for _ in range(max(1, args.stage_runs))]
    ms = {k: statistics.median(r[k] for r in runs) for k in runs[0]}
    torch.cuda.synchronize()
    print(json.dumps({"workload": "stages", "batch_pairs": B, "degree": n, "moduli": nmod, "plan": mult.plan,
                      "rns_tensor": args.rns_tensor, "runs": len(runs), "stage_ms": ms}), flush=True)


def run_codec(args):
    """Plaintext side at N = 2^14, L = 6, 64 vectors: SIMD encoding into the
    plaintext's Ntt polynomial, ciphertext x plaintext, decryption with SIMD
    decoding, and the expansion of seeded c1 polynomials, each a batched call
    on device-resident data."""
    import torch

    import __graft_entry__ as ge
    from oracle import ora

    ge.build()
    fg = ge.load_package()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    B = args.batch
    par_o, sk_o, _, cts, lhs, _ = make_inputs(ora, B)
    par = fg.BfvParameters(N, par_o.moduli, T)
    sk = fg.SecretKey(par, sk_o.coeffs)
    rng = np.random.default_rng(4)
    vals = rng.integers(0, T, (B, N), dtype=np.uint64)
    vals_d, ct_d = fg.to_device(vals), fg.to_device(lhs)
    pt = fg.plaintext_encode(par, 0, vals_d)
    prod = fg.ciphertext_mul_plain(par, 0, ct_d, pt)
    dec = sk.decrypt(ct_d)
    torch.cuda.synchronize()
    # Parity gate against the oracle on two entries.
    ctx = par_o.context_at_level(0)
    for b in (0, B - 1):
        m = ora.Poly.from_u64(ctx, ora.Plaintext.encode(vals[b], "simd", par_o).value).into_ntt()
        if not np.array_equal(fg.to_host(pt[b]), m.coefficients):
            raise SystemExit("bench: encoding is not bit-exact with the oracle")
        ct_o = ora.Ciphertext.from_array(par_o, lhs[b], 0)
        want = np.stack([(ct_o[k] * m).coefficients for k in range(2)])
        if not np.array_equal(fg.to_host(prod[b]), want):
            raise SystemExit("bench: ciphertext x plaintext is not bit-exact with the oracle")
        if not np.array_equal(fg.to_host(dec[b]), sk_o.decrypt(ct_o).decode("simd")):
            raise SystemExit("bench: decryption is not bit-exact with the oracle")
    # c1 of B seeded fresh ciphertexts (Poly::random_from_seed, rq/mod.rs:239-257).
    seeds = rng.integers(0, 256, (B, 32), dtype=np.uint8)
    seeds_d = torch.tensor(seeds, device=ct_d.device)
    ctx_d = par.context_at_level(0)
    c1 = fg.random_from_seed(ctx_d, seeds_d)
    if not np.array_equal(fg.to_host(c1[0]), ora.random_from_seed(ctx, bytes(seeds[0]))):
        raise SystemExit("bench: seeded expansion is not bit-exact with the oracle")
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    launches0 = fg.kernel_launch_count()
    with ClockSampler(0) as clocks:
        enc_ms = timed(lambda: fg.plaintext_encode(par, 0, vals_d))
        mul_ms = timed(lambda: fg.ciphertext_mul_plain(par, 0, ct_d, pt))
        dec_ms = timed(lambda: sk.decrypt(ct_d))
        seed_ms = timed(lambda: fg.random_from_seed(ctx_d, seeds_d, out=c1))
    launches = fg.kernel_launch_count() - launches0
    line = {"metric": "BFV plaintext side per second N=2^14 L=6 (SIMD encode, ct x pt, decrypt + decode)",
            "value": B / (dec_ms / 1000.0), "unit": "decryptions/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": enc_ms + mul_ms + dec_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic (seeded encryptions by the CPU oracle)",
            "config": {"workload": "codec", "degree": N, "moduli": L, "plaintext": T, "batch": B},
            "encode_per_s": B / (enc_ms / 1000.0), "mul_plain_per_s": B / (mul_ms / 1000.0),
            "decrypt_per_s": B / (dec_ms / 1000.0), "seeded_c1_per_s": B / (seed_ms / 1000.0),
            "seeded_c1_gbs_written": B * L * N * 8 / (seed_ms * 1e6),
            "gpu_launches": int(launches), "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)


def run_compose(args):
    """Compositions at N = 2^14, L = 6: inner sum of 16 ciphertexts (13 column
    rotations and the row rotation each), oblivious expansion of one
    ciphertext into 64, 4 dot products over 64 ciphertext-plaintext pairs, and
    the RGSW external product of 16 ciphertexts."""
    import torch

    import __graft_entry__ as ge
    from oracle import ora

    ge.build()
    fg = ge.load_package()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    rng = np.random.default_rng(33)
    par_o = ora.BfvParameters(N, T, moduli_sizes=[62] * L)
    sk = ora.SecretKey.random(par_o, rng)
    par = fg.BfvParameters(N, par_o.moduli, T)

    # One key per exponent: the inner sum's column rotation by N/4 uses
    # exponent 3^(N/4) = N + 1 mod 2N, the first expansion exponent.
    made = {}

    def keys(exps):
        for e in exps:
            if e not in made:
                g = ora.GaloisKey(sk, e, 0, 0, rng)
                made[e] = (g, fg.GaloisKey(par, e, g.ksk.c0_array(), g.ksk.c1_array()))
        return [made[e][0] for e in exps], [made[e][1] for e in exps]

    sum_exps = ora.EvaluationKey.inner_sum_exponents(par_o)
    exp_exps = ora.EvaluationKey.expansion_exponents(par_o, 6)
    sum_o, sum_k = keys(sum_exps)
    exp_o, exp_k = keys(exp_exps)
    cts = [sk.encrypt(ora.Plaintext.encode(rng.integers(0, T, N, dtype=np.uint64), "simd", par_o), rng)
           for _ in range(16)]
    arr = fg.to_device(np.stack([c.to_array() for c in cts]))
    ek = ora.EvaluationKey(sk, rng)
    ek.gk = dict(zip(sum_exps + exp_exps, sum_o + exp_o))
    # Parity gate.
    got = fg.to_host(fg.inner_sum(par, sum_k, arr[:1]))[0]
    if not np.array_equal(got, ek.computes_inner_sum(cts[0]).to_array()):
        raise SystemExit("bench: inner sum is not bit-exact with the oracle")
    got = fg.to_host(fg.expand(par, exp_k, arr[0], 4))
    want = ek.expands(cts[0], 4)
    if not all(np.array_equal(got[i], want[i].to_array()) for i in range(4)):
        raise SystemExit("bench: expansion is not bit-exact with the oracle")
    # RGSW external product (rgsw_ciphertext.rs:123-153) of the 16 ciphertexts.
    rg_o = ora.RGSWCiphertext(sk, ora.Plaintext.encode(rng.integers(0, T, N, dtype=np.uint64), "simd", par_o), rng)
    rg = fg.RGSWCiphertext(par, rg_o.ksk0.c0_array(), rg_o.ksk0.c1_array(), rg_o.ksk1.c0_array(),
                           rg_o.ksk1.c1_array())
    if not np.array_equal(fg.to_host(rg.external_product(arr[:1]))[0], rg_o.external_product(cts[0]).to_array()):
        raise SystemExit("bench: external product is not bit-exact with the oracle")
    ext_out = torch.empty_like(arr)
    groups, count = 4, 64
    db = fg.plaintext_encode(par, 0, fg.to_device(rng.integers(0, T, (count, N), dtype=np.uint64)))
    q = arr[torch.arange(groups * count, device=arr.device) % 16].reshape(groups, count, 2, L, N).contiguous()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    launches0 = fg.kernel_launch_count()
    with ClockSampler(0) as clocks:
        sum_ms = timed(lambda: fg.inner_sum(par, sum_k, arr))
        exp_ms = timed(lambda: fg.expand(par, exp_k, arr[0], 64))
        dot_ms = timed(lambda: fg.dot_product_scalar(par, 0, q, db))
        ext_ms = timed(lambda: rg.external_product(arr, out=ext_out))
    launches = fg.kernel_launch_count() - launches0
    line = {"metric": "BFV compositions N=2^14 L=6 (inner sum, expansion, dot product, RGSW product)",
            "value": 16 / (sum_ms / 1000.0), "unit": "inner sums/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": sum_ms + exp_ms + dot_ms + ext_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic (seeded encryptions and keys by the CPU oracle)",
            "config": {"workload": "compose", "degree": N, "moduli": L, "inner_sum_batch": 16,
                       "expansion_size": 64, "dot_products": groups, "dot_product_terms": count,
                       "external_products": 16},
            "inner_sum_ms": sum_ms, "expansion_64_ms": exp_ms, "dot_products_ms": dot_ms,
            "external_products_16_ms": ext_ms, "external_products_per_s": 16 / (ext_ms / 1000.0),
            "rotations_per_s": 16 * len(sum_exps) / (sum_ms / 1000.0),
            "gpu_launches": int(launches), "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)


def run_serialize(args):
    """Wire format: the Rq coefficient payload of 128 polynomials (64
    ciphertexts) at N = 2^14 with six 62-bit moduli, packed and unpacked on
    the device, in the power basis (pure bit packing, HBM-bound) and from the
    Ntt representation (with the NTTs the conversion needs)."""
    import torch

    import __graft_entry__ as ge
    from oracle import ora

    ge.build()
    fg = ge.load_package()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    moduli, ub = [], 1 << 62
    while len(moduli) < L:
        ub = ora.generate_prime(62, 2 * N, ub)
        moduli.append(ub)
    ctx = fg.Context(moduli, N)
    octx = ora.Context(moduli, N)
    rng = np.random.default_rng(5)
    polys = 128
    x = np.stack([rng.integers(0, m, N, dtype=np.uint64) for m in moduli])
    xd = fg.to_device(np.tile(x[None], (polys, 1, 1)))
    payload = fg.serialize(ctx, xd, 0)
    if bytes(payload[0].cpu().numpy().tobytes()) != ora.rq_payload(ora.Poly(octx, x.copy(), ora.POWER_BASIS)):
        raise SystemExit("bench: serialization is not byte-exact with the oracle")
    if not np.array_equal(fg.to_host(fg.deserialize(ctx, payload, 0)[:1])[0], x):
        raise SystemExit("bench: deserialization does not invert serialization")
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    out = fg.empty((polys, L, N))
    launches0 = fg.kernel_launch_count()
    with ClockSampler(0) as clocks:
        pack_ms = timed(lambda: fg.serialize(ctx, xd, 0))
        unpack_ms = timed(lambda: fg.deserialize(ctx, payload, 0))
        pack_ntt_ms = timed(lambda: fg.serialize(ctx, xd, 1))
        unpack_ntt_ms = timed(lambda: fg.deserialize(ctx, payload, 1))
    launches = fg.kernel_launch_count() - launches0
    words = polys * L * N * 8
    pb = payload.numel()
    pack_gbs = (words + pb) / (pack_ms / 1000) / 1e9
    unpack_gbs = (words + pb) / (unpack_ms / 1000) / 1e9
    peak, kind = _peaks()
    line = {"metric": "Rq payload pack/unpack GB/s N=2^14 L=6 (power basis)", "value": pack_gbs, "unit": "GB/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": pack_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
            "data": "synthetic", "config": {"workload": "serialize", "degree": N, "moduli": L, "polys": polys,
                                            "payload_bytes_per_poly": pb // polys},
            "roofline": {"bound": "hbm", "achieved": pack_gbs, "peak": peak, "unit": "GB/s", "frac": pack_gbs / peak,
                         "traffic": None, "kernel": "k_pack", "peak_kind": kind},
            "unpack_gbs": unpack_gbs, "pack_ms": pack_ms, "unpack_ms": unpack_ms,
            "pack_from_ntt_ms": pack_ntt_ms, "unpack_to_ntt_ms": unpack_ntt_ms,
            "gpu_launches": int(launches), "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)


def measure_ntt_degrees(fg, ora, torch, logns=(13, 15, 16), polys: int = 256, reps: int = 10):
    """Forward + inverse NTT of `polys` polynomials of six 62-bit moduli at
    each degree, under the default plan of the degree (device resident; the
    first polynomial checked against the oracle): GB/s of algorithmic traffic
    (each residue read and written once per transform, plus the twiddles)."""
    out = {}
    stream = torch.cuda.current_stream()
    start, mid, end = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    for logn in logns:
        n = 1 << logn
        moduli, ub = [], 1 << 62
        while len(moduli) < L:
            ub = ora.generate_prime(62, 2 * n, ub)
            moduli.append(ub)
        rng = np.random.default_rng(logn)
        one = np.stack([rng.integers(0, m, n, dtype=np.uint64) for m in moduli])
        ctx = fg.Context(moduli, n)
        buf = fg.to_device(np.tile(one[None], (polys, 1, 1)))
        expect = one.copy()
        for i, m in enumerate(moduli):
            ora.ntt_operator(m, n).forward(expect[i])
        fg.ntt_forward(ctx, buf)
        torch.cuda.synchronize()
        if not np.array_equal(fg.to_host(buf[:1])[0], expect):
            raise SystemExit(f"bench: NTT at 2^{logn} is not bit-exact with the oracle")
        fg.ntt_backward(ctx, buf)
        for _ in range(3):
            fg.ntt_forward(ctx, buf)
            fg.ntt_backward(ctx, buf)
        fwd = inv = 0.0
        for _ in range(reps):
            start.record(stream)
            fg.ntt_forward(ctx, buf)
            mid.record(stream)
            fg.ntt_backward(ctx, buf)
            end.record(stream)
            torch.cuda.synchronize()
            fwd += start.elapsed_time(mid)
            inv += mid.elapsed_time(end)
        fwd, inv = fwd / reps, inv / reps
        nbytes = 2 * 8 * polys * L * n + 2 * 8 * L * n
        out[f"2^{logn}"] = {"fwd_gbs": nbytes / (fwd / 1000) / 1e9, "inv_gbs": nbytes / (inv / 1000) / 1e9,
                            "fwd_ms": fwd, "inv_ms": inv, "block_logn": fg.ntt_plan_get(logn),
                            "cluster": fg.ntt_cluster_get(logn),
                            "fwd_butterflies_per_s": polys * L * butterflies_per_transform(logn) / (fwd / 1000)}
        del buf
    return out


def run_ntt(args):
    """The batched NTT configuration: forward + inverse over `--polys`
    polynomials of six 62-bit moduli at N = 2^logn (device resident), GB/s of
    algorithmic traffic against the measured HBM bandwidth. Every valid NTT
    plan is timed; the line reports the fastest (what fheg_ntt_autotune
    installs) and lists the others."""
    import torch

    import __graft_entry__ as ge
    from oracle import ora

    ge.build()
    fg = ge.load_package()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    logn = args.logn
    n = 1 << logn
    moduli, ub = [], 1 << 62
    while len(moduli) < L:
        ub = ora.generate_prime(62, 2 * n, ub)
        moduli.append(ub)
    rng = np.random.default_rng(1)
    polys = args.polys
    one = np.stack([rng.integers(0, m, n, dtype=np.uint64) for m in moduli])
    ctx = fg.Context(moduli, n)
    buf = fg.to_device(np.tile(one[None], (polys, 1, 1)))
    expect = one.copy()
    for i, m in enumerate(moduli):
        ora.ntt_operator(m, n).forward(expect[i])
    blocks = [bl for bl in (12, 13, 14) if bl <= logn and logn - bl <= 4 and (bl < logn or logn <= 14)] or [logn]
    # (block size, cluster mode): the 2^12-block plans also run as one pass on
    # clusters of the limb's blocks.
    plans = [(bl, False) for bl in blocks] + [(12, True) for bl in blocks if bl == 12 and logn > 12]
    default, default_cluster = fg.ntt_plan_get(logn), fg.ntt_cluster_get(logn)
    stream = torch.cuda.current_stream()
    start, mid, end = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    nbytes = 2 * 8 * polys * L * n + 2 * 8 * L * n
    results = {}
    launches = 0
    for bl, cluster in plans:
        fg.ntt_plan_set(logn, bl)
        fg.ntt_cluster_set(logn, cluster)
        fg.ntt_forward(ctx, buf)
        torch.cuda.synchronize()
        if not np.array_equal(fg.to_host(buf[:1])[0], expect):
            raise SystemExit(f"bench: NTT (blocks of 2^{bl}, cluster {cluster}) is not bit-exact with the oracle")
        fg.ntt_backward(ctx, buf)
        for _ in range(args.warmup):
            fg.ntt_forward(ctx, buf)
            fg.ntt_backward(ctx, buf)
        fwd = inv = 0.0
        launches0 = fg.kernel_launch_count()
        with ClockSampler(0) as clocks:
            for _ in range(args.steps):
                start.record(stream)
                fg.ntt_forward(ctx, buf)
                mid.record(stream)
                fg.ntt_backward(ctx, buf)
                end.record(stream)
                torch.cuda.synchronize()
                fwd += start.elapsed_time(mid)
                inv += mid.elapsed_time(end)
        fwd /= args.steps
        inv /= args.steps
        results[(bl, cluster)] = {"fwd_ms": fwd, "inv_ms": inv, "gbs": 2 * nbytes / ((fwd + inv) / 1000.0) / 1e9,
                                  "clocks": clocks.summary(), "launches": fg.kernel_launch_count() - launches0}
    fg.ntt_plan_set(logn, default)
    fg.ntt_cluster_set(logn, default_cluster)
    best = max(results, key=lambda k: results[k]["gbs"])
    r = results[best]
    fwd, inv, gbs = r["fwd_ms"], r["inv_ms"], r["gbs"]
    peak, kind = _peaks()
    line = {"metric": f"NTT fwd+inv GB/s N=2^{logn} L=6", "value": gbs, "unit": "GB/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": fwd + inv, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
            "config": {"workload": "ntt_batched", "degree": n, "moduli": L, "polys": polys, "block_logn": best[0],
                       "cluster": best[1],
                       "l2": f"buffer {polys * L * n * 8 / 1e6:.0f} MB > L2"},
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                         "traffic": None, "peak_kind": kind, "fwd_ms": fwd, "inv_ms": inv,
                         "fwd_gbs": nbytes / (fwd / 1000) / 1e9, "inv_gbs": nbytes / (inv / 1000) / 1e9},
            "plans": {f"{k[0]}{'-cluster' if k[1] else ''}": {"fwd_ms": v["fwd_ms"], "inv_ms": v["inv_ms"],
                                                               "gbs": v["gbs"]} for k, v in results.items()},
            "gpu_launches": int(r["launches"]), "clocks": r["clocks"]}
    print(json.dumps(line), flush=True)


def measure_intpeak(fg, torch, kinds=(0, 1, 2, 3, 4, 5), steps=5):
    """Operations per second of each integer probe (fheg_intpeak): 8 CTAs of
    256 threads per SM, four waves; CUDA events on the launching stream."""
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    blocks = props.multi_processor_count * 8 * 4
    sink = fg.empty((blocks * 256,))
    stream = torch.cuda.current_stream()
    out = {}
    for kind in kinds:
        iters = 2048 if kind >= 4 else 16384
        fg.intpeak_launch(kind, blocks, iters, sink)  # warm-up
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        start.record(stream)
        ops = sum(fg.intpeak_launch(kind, blocks, iters, sink) for _ in range(steps))
        end.record(stream)
        torch.cuda.synchronize()
        ms = start.elapsed_time(end)
        out[kind] = {"op": fg.INTPEAK_KINDS[kind], "ops_per_s": ops / (ms / 1000.0), "ms": ms / steps}
    return out, props.multi_processor_count


def butterflies_per_transform(logn: int) -> int:
    """Butterflies of one negacyclic NTT of 2^logn residues: N/2 per stage."""
    return (1 << logn) // 2 * logn


def run_intpeak(args):
    """Integer-throughput ceilings of this GPU: the 32-bit multiply forms the
    residue products are built from, 32-bit additions, and the NTT's 64-bit
    butterflies on register-resident values. Reported per second, per SM
    and clock (with the sampled SM clock), and set against what the NTT
    needs for 60% of the measured HBM bandwidth and what it reaches (forward
    NTT of 256 polynomials x 6 limbs at N = 2^logn, the default plan)."""
    import torch

    import __graft_entry__ as ge
    from oracle import ora

    ge.build()
    fg = ge.load_package()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    with ClockSampler(0) as clocks:
        probes, sms = measure_intpeak(fg, torch, steps=max(args.steps // 4, 3))
    clk = clocks.summary()
    mhz = clk["sm_mhz"] or 2070.0
    for v in probes.values():
        v["per_sm_per_clock"] = v["ops_per_s"] / (sms * mhz * 1e6)
    # The forward NTT as the ntt workload times it.
    logn = args.logn
    n = 1 << logn
    moduli, ub = [], 1 << 62
    while len(moduli) < L:
        ub = ora.generate_prime(62, 2 * n, ub)
        moduli.append(ub)
    ctx = fg.Context(moduli, n)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(1)
    q = torch.tensor([int(m) for m in moduli], dtype=torch.int64, device="cuda").view(1, L, 1)
    buf = torch.randint(0, 1 << 62, (args.polys, L, n), dtype=torch.int64, device="cuda", generator=gen) % q
    for _ in range(3):
        fg.ntt_forward(ctx, buf)
        fg.ntt_backward(ctx, buf)
    stream = torch.cuda.current_stream()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    start.record(stream)
    for _ in range(args.steps):
        fg.ntt_forward(ctx, buf)
    end.record(stream)
    torch.cuda.synchronize()
    fwd_ms = start.elapsed_time(end) / args.steps
    limbs = args.polys * L
    bfly = limbs * butterflies_per_transform(logn)
    nbytes = 16 * limbs * n
    peak, kind = _peaks()
    need = 0.6 * peak * 1e9 / nbytes * bfly  # butterflies/s for 60% of HBM
    fwd_bps = bfly / (fwd_ms / 1000.0)
    ceiling = probes[4]["ops_per_s"]
    line = {"metric": "integer throughput ceilings (ops/s)", "value": ceiling, "unit": "butterflies/s",
            "n_gpus": 1, "steps": args.steps, "warmup": 1, "higher_is_better": True, "dtype": "u64",
            "data": "synthetic", "config": {"workload": "intpeak", "sms": sms, "threads_per_sm": 2048},
            "probes": {str(k): v for k, v in probes.items()},
            "ntt": {"degree": n, "limbs": limbs, "fwd_ms": fwd_ms, "fwd_gbs": nbytes / (fwd_ms / 1000.0) / 1e9,
                    "fwd_butterflies_per_s": fwd_bps, "frac_of_butterfly_ceiling": fwd_bps / ceiling,
                    "hbm_frac": nbytes / (fwd_ms / 1000.0) / 1e9 / peak,
                    "butterflies_per_s_for_60pct_hbm": need, "ceiling_over_need": ceiling / need,
                    "peak_kind": kind},
            "clocks": clk}
    print(json.dumps(line), flush=True)


def measure_rotations(fg, ora, torch, count: int, steps: int, warmup: int, ntt_block: str = "auto",
                      ntt_cluster: str = "default"):
    """Uneven-level rotation batch: N = 2^15, twelve 62-bit moduli at the top
    level, `count` ciphertexts each switched to a random level (4 to 12 live
    moduli) and rotated by a random column step in [1, N/2) with the Galois
    key of its (step, level); ~1 GB of keys resident at 32. One step = the
    whole ragged batch in one call (one launch per stage). The first and last
    rotation are checked against the oracle before timing."""
    n, top = 1 << 15, 12
    if ntt_cluster != "default":
        fg.ntt_cluster_set(15, ntt_cluster == "on")
    rng = np.random.default_rng(15)
    par_o = ora.BfvParameters(n, T, moduli_sizes=[62] * top)
    par = fg.BfvParameters(n, par_o.moduli, T)
    sk = ora.SecretKey.random(par_o, rng)
    levels = [int(x) for x in rng.integers(0, top - 3, count)]  # 4..12 live moduli
    rot_steps = [int(x) for x in rng.integers(1, n // 2, count)]
    keys, gks_o, cts_o, cts_d = [], [], [], []
    key_bytes = 0
    for b in range(count):
        e = ora.rotation_exponent(par_o, rot_steps[b])
        gk = ora.GaloisKey(sk, e, levels[b], levels[b], rng)
        gks_o.append(gk)
        c0, c1 = gk.ksk.c0_array(), gk.ksk.c1_array()
        key_bytes += c0.nbytes + c1.nbytes
        keys.append(fg.GaloisKey(par, e, c0, c1, levels[b], levels[b]))
        v = rng.integers(0, T, n, dtype=np.uint64)
        ct = sk.encrypt(ora.Plaintext.encode(v, "simd", par_o, levels[b]), rng)
        cts_o.append(ct)
        cts_d.append(fg.to_device(ct.to_array()))
    outs = [fg.empty(c.shape) for c in cts_d]
    if ntt_block == "auto":
        fg.ntt_autotune(par.context_at_level(0), 64)
    else:
        fg.ntt_plan_set(15, int(ntt_block))
    fg.rotate_batch(par, keys, cts_d, outs)
    torch.cuda.synchronize()
    for b in (0, count - 1):
        if not np.array_equal(fg.to_host(outs[b]), gks_o[b].relinearize(cts_o[b]).to_array()):
            raise SystemExit(f"bench: rotation {b} is not bit-exact with the oracle")
    for _ in range(warmup):
        fg.rotate_batch(par, keys, cts_d, outs)
    stream = torch.cuda.current_stream()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    launches0 = fg.kernel_launch_count()
    start.record(stream)
    for _ in range(steps):
        fg.rotate_batch(par, keys, cts_d, outs)
    end.record(stream)
    torch.cuda.synchronize()
    launches = fg.kernel_launch_count() - launches0
    ms = start.elapsed_time(end) / steps
    # One rotation per call (GaloisKey::relinearize on each ciphertext).
    start.record(stream)
    for b in range(count):
        keys[b].relinearize(cts_d[b][None])
    end.record(stream)
    torch.cuda.synchronize()
    single_ms = start.elapsed_time(end)
    return {"value": count / (ms / 1000), "unit": "ct/s", "ms_per_step": ms, "steps": steps,
            "config": {"workload": "rotation_uneven_levels", "degree": n, "top_moduli": top, "count": count,
                       "live_moduli": [top - l for l in levels], "key_bytes_resident": key_bytes,
                       "ntt_block_logn": fg.ntt_plan_get(15)},
            "single": {"value": count / (single_ms / 1000), "unit": "ct/s", "note": "one call per ciphertext"},
            "batch_vs_single": single_ms / ms, "gpu_launches": int(launches)}


def run_rotate(args):
    """The uneven-level rotation batch (measure_rotations) as its own line."""
    import torch

    import __graft_entry__ as ge
    from oracle import ora

    ge.build()
    fg = ge.load_package()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    with ClockSampler(0) as clocks:
        r = measure_rotations(fg, ora, torch, args.rot_count, args.steps, args.warmup, args.ntt_block,
                              args.ntt_cluster)
    line = {"metric": "ragged rotation ct/s N=2^15 L=4..12 (GaloisKey per level)", "value": r["value"],
            "unit": "ct/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic (seeded encryptions and keys by the CPU oracle)", "config": r["config"],
            "single": r["single"], "batch_vs_single": r["batch_vs_single"], "gpu_launches": r["gpu_launches"],
            "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)


SERVE_SETS = [(1 << 13, 3), (1 << 14, 6), (1 << 15, 12)]
SERVE_MIX = (("mul", 0.50), ("rot", 0.30), ("add", 0.15), ("down", 0.05))


def _serve_setup(fg, ora, torch, n, nm, seed, ring):
    """Keys, pinned input ciphertexts and a pinned output ring of one
    parameter set, at every level with at least two live moduli (relinearization
    key, multiplicator and two Galois keys per level)."""
    rng = np.random.default_rng(seed)
    par_o = ora.BfvParameters(n, T, moduli_sizes=[62] * nm)
    sk = ora.SecretKey.random(par_o, rng)
    par = fg.BfvParameters(n, par_o.moduli, T)

    def pinned(shape):
        return torch.empty(shape, dtype=torch.int64, pin_memory=True).numpy().view(np.uint64)

    levels = []
    for lvl in range(nm - 1):
        rk_o = ora.RelinearizationKey(sk, rng, lvl, lvl)
        rk = fg.RelinearizationKey(par, rk_o.ksk.c0_array(), rk_o.ksk.c1_array(), lvl, lvl)
        exps = (2 * n - 1, ora.rotation_exponent(par_o, 1 + lvl))
        gks_o = [ora.GaloisKey(sk, e, lvl, lvl, rng) for e in exps]
        gks = [fg.GaloisKey(par, e, g.ksk.c0_array(), g.ksk.c1_array(), lvl, lvl) for e, g in zip(exps, gks_o)]
        cts_o = [sk.encrypt(ora.Plaintext.encode(rng.integers(0, T, n, dtype=np.uint64), "simd", par_o, lvl), rng)
                 for _ in range(3)]
        cts = []
        for c in cts_o:
            h = pinned((2, nm - lvl, n))
            h[...] = c.to_array()
            cts.append(h)
        levels.append({"rk_o": rk_o, "rk": rk, "mult": fg.Multiplicator.default(rk), "gks_o": gks_o, "gks": gks,
                       "cts_o": cts_o, "cts": cts})
    slot_words = 2 * nm * n
    return {"n": n, "L": nm, "par_o": par_o, "par": par, "levels": levels, "ring": ring,
            "out_flat": pinned((ring * slot_words,)), "slot_words": slot_words}


def _serve_requests(count, seed):
    """(set index, kind, level, operand a, operand b, key index) of each
    request: set uniform, kind by the mix, level uniform over the live range."""
    rng = np.random.default_rng(seed)
    kinds = [k for k, _ in SERVE_MIX]
    probs = [p for _, p in SERVE_MIX]
    sets = rng.integers(0, len(SERVE_SETS), count)
    ks = rng.choice(len(kinds), count, p=probs)
    lv = [int(rng.integers(0, SERVE_SETS[si][1] - 1)) for si in sets]
    a, b, g = rng.integers(0, 3, count), rng.integers(0, 3, count), rng.integers(0, 2, count)
    return [(int(sets[i]), kinds[ks[i]], lv[i], int(a[i]), int(b[i]), int(g[i])) for i in range(count)]


def _serve_out(s, slot, shape):
    w = int(np.prod(shape))
    k = slot % s["ring"]
    return s["out_flat"][k * s["slot_words"]:k * s["slot_words"] + w].reshape(shape)


def _serve_submit(srv, setups, req, slot):
    si, kind, lvl, a, b, g = req
    s = setups[si]
    lv = s["levels"][lvl]
    n, live = s["n"], s["L"] - lvl
    if kind == "mul":
        return srv.submit_mul_relin(lv["mult"], lv["cts"][a], lv["cts"][b], out=_serve_out(s, slot, (2, live, n)))
    if kind == "rot":
        return srv.submit_rotate(lv["gks"][g], lv["cts"][a], out=_serve_out(s, slot, (2, live, n)))
    if kind == "add":
        return srv.submit_add(s["par"], lvl, lv["cts"][a], lv["cts"][b], out=_serve_out(s, slot, (2, live, n)))
    return srv.submit_switch_down(s["par"], lvl, lv["cts"][a], out=_serve_out(s, slot, (2, live - 1, n)))


def _serve_run(fg, setups, reqs, budget, streams, max_batch, arrivals=None):
    """Submits `reqs` (all at once, or at the `arrivals` offsets in seconds)
    and returns (requests/s, latencies in ms, batches)."""
    with fg.Server(budget, streams=streams, max_batch=max_batch) as srv:
        ids = []
        t0 = time.perf_counter()
        for i, r in enumerate(reqs):
            if arrivals is not None:
                target = t0 + arrivals[i]
                while True:
                    left = target - time.perf_counter()
                    if left <= 0:
                        break
                    if left > 3e-4:
                        time.sleep(left - 2e-4)
            ids.append(_serve_submit(srv, setups, r, i))
        for rid in ids:
            srv.wait(rid, 600000)
        times = np.array([srv.times(rid) for rid in ids], dtype=np.int64)
        batches = srv.stats()["batches"]
    lat = (times[:, 2] - times[:, 0]) / 1e6
    span = (times[:, 2].max() - times[:, 0].min()) / 1e9
    return len(reqs) / span, lat, batches


def run_serve(args):
    """Serving loop: a stream of requests over three parameter sets (N = 2^13
    with 3 moduli, 2^14 with 6, 2^15 with 12, chosen uniformly), 50% mul+relin,
    30% rotation, 15% addition and 5% switch-down, keys resident, ciphertexts
    in pinned host memory. The continuous-batching server (HBM budget, several
    streams) against the same server restricted to one request at a time:
    saturation throughput with everything submitted at once, and p50/p99
    latency under Poisson arrivals at 70% of the one-at-a-time capacity and at
    70% of the batched capacity."""
    import torch

    import __graft_entry__ as ge
    from oracle import ora

    ge.build()
    fg = ge.load_package()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    fg.rns_tensor_set(args.rns_tensor == "on")
    ring = 64
    setups = [_serve_setup(fg, ora, torch, n, nm, 100 + k, ring) for k, (n, nm) in enumerate(SERVE_SETS)]
    budget = int(args.serve_budget_gb * (1 << 30))
    for s in setups:
        fg.ntt_autotune(s["par"].context_at_level(0), 32)
        for lv in s["levels"]:
            lv["mult"].autotune(4)   # the small-batch plan
            lv["mult"].autotune(32)  # the plan of full batches
    # Parity gate: every operation of every set, at its top and bottom live
    # levels, through the server alone, against the oracle.
    with fg.Server(budget, streams=1, max_batch=1) as srv:
        for si, s in enumerate(setups):
            for lvl in (0, s["L"] - 2):
                lv = s["levels"][lvl]
                co = lv["cts_o"]
                checks = [(("mul", 0, 1, 0), ora.Multiplicator.default(lv["rk_o"]).multiply(co[0], co[1])),
                          (("rot", 2, 0, 1), lv["gks_o"][1].relinearize(co[2])),
                          (("add", 1, 2, 0), co[1] + co[2]),
                          (("down", 0, 0, 0), co[0].copy().switch_down())]
                for (kind, a, b, g), want in checks:
                    got = srv.wait(_serve_submit(srv, setups, (si, kind, lvl, a, b, g), 0), 600000).copy()
                    if not np.array_equal(got, want.to_array()):
                        raise SystemExit(f"bench: served {kind} at N={s['n']} level {lvl} is not bit-exact")
    reqs = _serve_requests(args.serve_requests, 7)
    warm = _serve_requests(min(200, args.serve_requests), 8)
    for _ in range(max(1, args.warmup // 2)):
        _serve_run(fg, setups, warm, budget, args.serve_streams, args.serve_batch)
        _serve_run(fg, setups, warm, budget, 1, 1)
    launches0 = fg.kernel_launch_count()
    with ClockSampler(0) as clocks:
        thr_b, lat_sat_b, batches_b = _serve_run(fg, setups, reqs, budget, args.serve_streams, args.serve_batch)
    launches = fg.kernel_launch_count() - launches0
    thr_1, lat_sat_1, _ = _serve_run(fg, setups, reqs, budget, 1, 1)
    rng = np.random.default_rng(9)
    gaps = rng.exponential(1.0, len(reqs))

    def poisson(rate, streams, max_batch):
        _, lat, batches = _serve_run(fg, setups, reqs, budget, streams, max_batch, np.cumsum(gaps) / rate)
        return {"offered_req_s": rate, "p50_ms": float(np.percentile(lat, 50)),
                "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean()), "batches": int(batches)}

    low = 0.7 * thr_1
    at_low_b = poisson(low, args.serve_streams, args.serve_batch)
    at_low_1 = poisson(low, 1, 1)
    high = 0.7 * thr_b
    at_high_b = poisson(high, args.serve_streams, args.serve_batch)
    h2d = d2h = 0
    for si, kind, lvl, _, _, _ in reqs:
        s = setups[si]
        live = s["L"] - lvl
        ct_bytes = 2 * live * s["n"] * 8
        h2d += ct_bytes * (2 if kind in ("mul", "add") else 1)
        d2h += ct_bytes if kind != "down" else 2 * (live - 1) * s["n"] * 8
    line = {"metric": "BFV serving req/s (mixed N=2^13..2^15), p50/p99 vs one-at-a-time",
            "value": thr_b, "unit": "req/s", "n_gpus": 1, "steps": 1, "warmup": args.warmup,
            "ms_per_step": 1000 * len(reqs) / thr_b, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded encryptions and keys by the CPU oracle)",
            "config": {"workload": "serve_mixed", "sets": [{"degree": n, "moduli": nm} for n, nm in SERVE_SETS],
                       "levels": "uniform over the live range (2 .. L moduli)",
                       "mix": dict(SERVE_MIX), "requests": len(reqs), "hbm_budget_bytes": budget,
                       "streams": args.serve_streams, "max_batch": args.serve_batch,
                       "ntt_block_logn": {str(n): fg.ntt_plan_get(n.bit_length() - 1) for n, _ in SERVE_SETS},
                       "host_buffers": "pinned"},
            "e2e": {"value": thr_b, "unit": "req/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "note": "one step = all requests, host buffers to host buffers"},
            "saturation": {"batched_req_s": thr_b, "one_at_a_time_req_s": thr_1, "speedup": thr_b / thr_1,
                           "batched_batches": int(batches_b)},
            "poisson_at_70pct_of_one_at_a_time": {"batched": at_low_b, "one_at_a_time": at_low_1},
            "poisson_at_70pct_of_batched": {"batched": at_high_b},
            "gpu_launches": int(launches), "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: 400 for the batched multiplication, about 1 s; 20 otherwise)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="mul_relin", choices=["mul_relin", "ntt", "rotate", "serve", "stages", "codec", "compose",
                                                             "serialize", "intpeak"])
    ap.add_argument("--rot-count", type=int, default=32)
    ap.add_argument("--polys", type=int, default=256)
    ap.add_argument("--logn", type=int, default=14)
    ap.add_argument("--moduli", type=int, default=L, help="stages workload: ciphertext moduli")
    ap.add_argument("--ntt-prefetch", default="off", choices=["on", "off"],
                    help="L2 prefetch of the next CTA's NTT input")
    ap.add_argument("--stage-plan", default="", help="A,C,D,F,F-split,D-split plan of the multiply stages")
    ap.add_argument("--ntt-block", default="auto", help="NTT plan for the degree: auto (autotune) or a block log2")
    ap.add_argument("--rns-tensor", default="on", choices=["on", "off"],
                    help="RNS scalings of the multiplication on the tensor cores (on) or the CUDA cores (off)")
    ap.add_argument("--stage-runs", type=int, default=1, help="stages workload: median over this many runs")
    ap.add_argument("--ntt-cluster", default="default", choices=["default", "on", "off"],
                    help="rotate workload: cluster mode of the 2^15 NTT plan")
    ap.add_argument("--serve-requests", type=int, default=2000)
    ap.add_argument("--serve-budget-gb", type=float, default=24.0)
    ap.add_argument("--serve-streams", type=int, default=4)
    ap.add_argument("--serve-batch", type=int, default=32)
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 400 if args.workload == "mul_relin" and args.impl == "ours" else 20
    if args.workload == "serve":
        # A server loads every kernel when CUDA starts: with lazy loading the
        # first launch of each kernel instantiation (parameter set, level,
        # batch size, plan) stalls the requests in flight for milliseconds,
        # which measured as a 2-9 ms p99 and up to 25% less throughput.
        os.environ.setdefault("CUDA_MODULE_LOADING", "EAGER")
    if args.ntt_prefetch == "on":
        import __graft_entry__ as ge

        ge.build()
        ge.load_package().ntt_prefetch_set(True)
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if args.workload == "ntt":
        run_ntt(args)
    elif args.workload == "rotate":
        run_rotate(args)
    elif args.workload == "serve":
        run_serve(args)
    elif args.workload == "stages":
        run_stages(args)
    elif args.workload == "codec":
        run_codec(args)
    elif args.workload == "compose":
        run_compose(args)
    elif args.workload == "serialize":
        run_serialize(args)
    elif args.workload == "intpeak":
        run_intpeak(args)
    elif args.impl == "reference":
        run_reference(args, rank)
    else:
        run_ours(args, rank, world)


if __name__ == "__main__":
    main()
