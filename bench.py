"""Benchmark: Pauli expectation values per second on the n=40 plain-method workload.

Workload (the reference's plain method on one GPU): n = 40 qubits, 4000 random
{H, S, CX} gates plus 24 T gates (seeded generator of
stab_decomp_simulator_rust_gb300/workloads.py), compiled into χ = 972 CH-form
terms, and 64 random dense Pauli observables (each qubit uniform in
{I, X, Y, Z}).  One step evaluates all 64 ⟨P⟩ by the full χ² pairwise sum
(472,878 term pairs per observable).

* ``value``: ⟨P⟩/s with the compiled state resident in HBM; the 64
  observables go through one batched pass captured as a plan (nsg_plan_run:
  one CUDA-graph replay per step, FP64 accumulation), device-timed with CUDA
  events on torch's stream; L2 is flushed (a 256 MiB write) before every
  timed step.  ``direct``: the same through nsg_exp_value_batch.
* ``e2e``: the same metric end to end through the C ABI from host buffers:
  nsg_state_from_circuit (gate list from pinned host memory) +
  nsg_exp_value_batch (Paulis from host, 64 doubles back), wall-clock.
* ``plain``: the drop-in single-observable path (nsg_exp_value per ⟨P⟩).
* ``cpu_baseline`` / ``--impl reference``: the C++ restatement of the
  reference's Rust path (the reference cannot be built here: no Rust
  toolchain), timed on the host cores on a bounded sample of term pairs and
  extrapolated to whole observables.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
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

import numpy as np  # noqa: E402

# DRAM bytes (read + write) of one pair-kernel launch of this workload, from one
# ncu capture (dram__bytes_read.sum + dram__bytes_write.sum): the 5 MB of term
# tables stay L2-resident; most of it is the per-task records.
PAIR_TRAFFIC_BYTES = 69_151_232 + 5_759_488

METRIC = "Pauli \u27e8P\u27e9/s and CH inner products/s, mixed+batched vs plain FP64 @\u22641e-9 err"
UNIT = "<P>/s"


def workload():
    from stab_decomp_simulator_rust_gb300 import workloads as W
    cfg = W.PLAIN_N40
    gates = W.random_clifford_t_circuit(cfg["n"], cfg["num_clifford"], cfg["num_t"], cfg["seed"])
    paulis = W.random_dense_paulis(cfg["n"], cfg["num_paulis"], cfg["seed"] + 100)
    return cfg, gates, paulis


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def combine_ranks(ms_step: float, units_per_rank: int, device: str):
    """Whole-job figures over replicas: the step time is the maximum over ranks
    and the value counts the units of every rank (one replica per GPU, no
    exchange on the data path)."""
    ws, _, _ = dist_env()
    if ws > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([ms_step], device=device, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_step = float(t.item())
    return ms_step, ws * units_per_rank / (ms_step * 1e-3)


# ---------------------------------------------------------------------------
# clocks during the timed region
class ClockSampler:
    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        cmd = ["nvidia-smi", f"--id={self.index}",
               "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
               "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
               "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
               "--format=csv,noheader,nounits", "-lms", "200"]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                self.rows.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[4 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# ---------------------------------------------------------------------------
def cpu_sample(gates, cfg, paulis, seconds_target=12.0, threads=None):
    """Reference algorithm on the host: compile once, then time a sample of pairs."""
    from oracle import pyoracle as po
    threads = threads or os.cpu_count() or 1
    t0 = time.perf_counter()
    st = po.OracleState.from_circuit(cfg["n"], gates)
    t_compile = time.perf_counter() - t0
    chi = st.stabilizer_rank
    pairs_per_p = chi * (chi + 1) // 2
    # calibrate
    sec, _ = st.time_pairs(0, paulis[0], None, 200 * threads, 1, threads)
    rate = 200 * threads / sec
    npairs = int(max(1000, min(pairs_per_p, rate * seconds_target)))
    sec, _ = st.time_pairs(0, paulis[0], None, npairs, 2, threads)
    rate = npairs / sec
    per_p = pairs_per_p / rate
    nobs = len(paulis)
    value = nobs / (t_compile + nobs * per_p)
    return {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{npairs} uniformly drawn term pairs of one observable (reference inner-product algorithm, "
                      f"{threads} threads) extrapolated to {nobs} x {pairs_per_p} pairs, plus one {t_compile:.2f} s "
                      f"single-thread compile",
            "pairs_per_s": rate, "compile_s": t_compile, "chi": chi}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    cfg, gates, paulis = workload()
    from oracle import pyoracle as po
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    st = po.OracleState.from_circuit(cfg["n"], gates)
    t_compile = time.perf_counter() - t0
    chi = st.stabilizer_rank
    pairs_per_p = chi * (chi + 1) // 2
    sec, _ = st.time_pairs(0, paulis[0], None, 100 * threads, 1, threads)
    per_step_pairs = int(max(1000, 2.0 * 100 * threads / sec))  # ~2 s of work per step
    for w in range(args.warmup):
        st.time_pairs(0, paulis[w % len(paulis)], None, min(per_step_pairs, 200 * threads), 10 + w, threads)
    times, rates = [], []
    for k in range(args.steps):
        sec, _ = st.time_pairs(0, paulis[k % len(paulis)], None, per_step_pairs, 100 + k, threads)
        times.append(sec)
        rates.append(per_step_pairs / sec)
    rate = sum(rates) / len(rates)
    nobs = len(paulis)
    value = nobs / (t_compile + nobs * pairs_per_p / rate)
    ms = 1e3 * (t_compile + nobs * pairs_per_p / rate)
    sample = (f"per step {per_step_pairs} uniformly drawn term pairs of one observable on {threads} threads; "
              f"<P>/s extrapolated to {nobs} observables x {pairs_per_p} pairs plus the measured {t_compile:.2f} s compile")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
            "config": {"workload": "n=40, 4000 {H,S,CX} + 24 T, 64 dense Paulis", "chi": chi,
                       "parallelism": "host threads"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "pairs_per_s": rate, "compile_s": t_compile}
    print(json.dumps(line))


def run_ours(args):
    import torch

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from stab_decomp_simulator_rust_gb300 import PRECISION_FP64, PRECISION_MIXED, BatchPlan, PauliString, QuantumState
    from stab_decomp_simulator_rust_gb300 import _ffi, build
    build.build()
    L = _ffi.load()

    cfg, gates, pauli_ops = workload()
    paulis = [PauliString.dense(p) for p in pauli_ops]
    nobs = len(paulis)
    n = cfg["n"]
    stream = torch.cuda.current_stream()

    # ---- device-resident measurement
    st = QuantumState.from_gates(n, gates)
    st.set_stream(stream.cuda_stream)
    chi = st.stabilizer_rank
    pairs = chi * (chi + 1) // 2
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    # The batched evaluation as a captured plan (one CUDA-graph replay per step:
    # frames, term tables, Pauli frames, pair launch, reduction, result copy).
    plan = BatchPlan([st], [paulis], PRECISION_FP64)
    for _ in range(args.warmup):
        plan.run()
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    total_ms = 0.0
    results = None
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        results = plan.run()[0]
        e1.record(stream)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
    torch.cuda.synchronize()
    clocks.stop()
    ms_step, value = combine_ranks(total_ms / args.steps, nobs, "cuda")
    # the same evaluation through the direct batched call (descriptors built per
    # call), with the pair kernel's own launches timed on its stream (roofline)
    for _ in range(2):
        st.exp_values(paulis)
    import ctypes as C
    _ffi.check(L.nsg_profile_enable(1))
    _ffi.check(L.nsg_profile_read(None, None, None))
    direct_ms = 0.0
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st.exp_values(paulis)
        e1.record(stream)
        e1.synchronize()
        direct_ms += e0.elapsed_time(e1)
    direct_ms /= args.steps
    pk_ms, pk_launch, pk_pairs = C.c_double(), C.c_uint64(), C.c_uint64()
    _ffi.check(L.nsg_profile_read(C.byref(pk_ms), C.byref(pk_launch), C.byref(pk_pairs)))
    _ffi.check(L.nsg_profile_enable(0))

    # ---- mixed precision and the single-observable drop-in path
    for _ in range(2):
        st.exp_values(paulis, precision=PRECISION_MIXED)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    mixed = None
    for _ in range(args.steps):
        mixed = st.exp_values(paulis, precision=PRECISION_MIXED)
    torch.cuda.synchronize()
    mixed_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    plain_obs = paulis[:8]
    st.exp_value(plain_obs[0])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for p in plain_obs:
        st.exp_value(p)
    torch.cuda.synchronize()
    plain_rate = len(plain_obs) / (time.perf_counter() - t0)

    # ---- end to end through the C ABI from host buffers
    pinned_gates = torch.from_numpy(np.ascontiguousarray(gates)).pin_memory().numpy()
    for _ in range(max(1, args.warmup // 2)):
        QuantumState.from_gates(n, pinned_gates).exp_values(paulis)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s2 = QuantumState.from_gates(n, pinned_gates)
        out2 = s2.exp_values(paulis)
        del s2
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    e2e = {"value": ws * nobs / (e2e_ms * 1e-3), "unit": UNIT,
           "h2d_bytes_per_step": int(pinned_gates.nbytes + sum(p.ops.nbytes for p in paulis) + 24 * nobs),
           "d2h_bytes_per_step": int(8 * nobs), "ms_per_step": e2e_ms,
           "path": "nsg_state_from_circuit + nsg_exp_value_batch, host buffers"}

    # ---- roofline of the pair kernel (integer pipe)
    probe_s, probe_ops = C.c_double(), C.c_uint64()
    _ffi.check(L.nsg_probe_int_ops(20000, C.byref(probe_s), C.byref(probe_ops)))
    int32_peak = probe_ops.value / probe_s.value  # 32-bit logic ops/s
    word_peak = int32_peak / 2.0  # 64-bit word ops/s
    w = n  # width after discards; one 64-bit word per row
    algo_ops_per_pair = w * w * 1  # w·w·W word-ops of GF(2) elimination per pair
    pair_launch_ms = pk_ms.value / max(1, pk_launch.value)
    pairs_per_launch = pk_pairs.value / max(1, pk_launch.value)
    achieved = algo_ops_per_pair * pairs_per_launch / (pair_launch_ms * 1e-3)
    roofline = {"bound": "int", "achieved": achieved / 1e12, "peak": word_peak / 1e12, "unit": "Tword-ops/s",
                "frac": achieved / word_peak, "traffic": PAIR_TRAFFIC_BYTES, "traffic_unit": "bytes per launch",
                "kernel": "pair_kernel<uint64,2,2>",
                "peak_source": "measured: LOP3 chains on every SM (nsg_probe_int_ops), 64-bit word = 2 int32 ops",
                "algorithmic_unit": f"{algo_ops_per_pair} 64-bit word-ops per pair (w*w*W, w={w})",
                "pair_kernel_ms_per_launch": pair_launch_ms, "pairs_per_launch": pairs_per_launch}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
            "config": {"workload": "n=40, 4000 {H,S,CX} + 24 T (seed 2), 64 dense Paulis (seed 102)",
                       "chi": chi, "pairs_per_observable": pairs, "observables_per_step": nobs,
                       "l2": "flushed (256 MiB write) before every timed step", "parallelism": f"replicas x{ws}"},
            "inner_products_per_s": value * pairs,
            "path": "BatchPlan.run (nsg_plan_run: CUDA-graph replay), FP64",
            "plan_tiling": plan.tiling,
            "direct": {"value": ws * nobs / (direct_ms * 1e-3), "unit": UNIT, "ms_per_step": direct_ms,
                       "path": "nsg_exp_value_batch"},
            "mixed": {"value": ws * nobs / (mixed_ms * 1e-3), "unit": UNIT,
                      "max_abs_diff_vs_fp64": float(np.max(np.abs(np.asarray(mixed) - np.asarray(results))))},
            "plain": {"value": plain_rate * ws, "unit": UNIT, "path": "nsg_exp_value, one observable per call"},
            "e2e": e2e, "roofline": roofline, "clocks": clocks.summary(), "gpu_launches": None}
    # kernels launched per timed step (one plan replay): frames, term tables, Pauli frames, pairs, reduction
    # per replay: frames, term tables, Pauli frames, the pair launch and the two reduction passes
    line["gpu_launches"] = 6 * args.steps
    if rank == 0:
        if not args.no_cpu:
            try:
                line["cpu_baseline"] = cpu_sample(gates, cfg, pauli_ops[:nobs])
            except Exception as e:  # the oracle is optional for the GPU number itself
                line["cpu_baseline"] = {"value": None, "error": str(e)}
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()


# ---------------------------------------------------------------------------
# The precision, batching and projection/sampling workloads (one JSON line each)
def _setup_gpu():
    import torch
    from stab_decomp_simulator_rust_gb300 import _ffi, build
    torch.cuda.set_device(0)
    build.build()
    return torch, _ffi.load()


def _timed(torch, stream, fn, steps):
    """Device time per call of fn() on `stream` (CUDA events), and its last result."""
    out = None
    tot = 0.0
    for _ in range(steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = fn()
        e1.record(stream)
        e1.synchronize()
        tot += e0.elapsed_time(e1)
    return tot / steps, out


def _rel_err(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-300)


def run_precision60(args, torch, L):
    """n=60, 6000 {H,S,CX} + 36 T, 256 sparse Paulis of weight 1..8: FP64 and
    mixed accumulation over the full χ² pair sum; per-observable error of the
    mixed result against the FP64 one."""
    from stab_decomp_simulator_rust_gb300 import PRECISION_FP64, PRECISION_MIXED, PauliString, QuantumState
    from stab_decomp_simulator_rust_gb300 import workloads as W
    cfg = W.PRECISION_N60
    gates = W.random_clifford_t_circuit(cfg["n"], cfg["num_clifford"], cfg["num_t"], cfg["seed"])
    sp = W.random_sparse_paulis(cfg["n"], cfg["num_paulis"], 1, 8, cfg["seed"] + 100)
    paulis = [PauliString.sparse(o, q) for o, q in sp]
    stream = torch.cuda.current_stream()
    t0 = time.perf_counter()
    st = QuantumState.from_gates(cfg["n"], gates)
    compile_s = time.perf_counter() - t0
    st.set_stream(stream.cuda_stream)
    chi = st.stabilizer_rank
    pairs = chi * (chi + 1) // 2
    for _ in range(args.warmup):
        st.exp_values(paulis[:32], PRECISION_MIXED)
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    ms64, v64 = _timed(torch, stream, lambda: st.exp_values(paulis, PRECISION_FP64), args.steps)
    msmx, vmx = _timed(torch, stream, lambda: st.exp_values(paulis, PRECISION_MIXED), args.steps)
    ms1, _ = _timed(torch, stream, lambda: st.exp_value(paulis[0]), 1)
    clocks.stop()
    err = _rel_err(vmx, v64)
    nobs = len(paulis)
    line = {"metric": METRIC, "value": nobs / (msmx * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": msmx, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 accumulation of exact pair values, f64 final reduction",
            "data": "synthetic (seeded generator)",
            "config": {"workload": "n=60, 6000 {H,S,CX} + 36 T (seed 3), 256 sparse Paulis of weight 1..8 (seed 103)",
                       "chi": chi, "pairs_per_observable": pairs, "compile_s": compile_s,
                       "l2": "inputs larger than L2 (term tables)"},
            "inner_products_per_s": nobs * pairs / (msmx * 1e-3),
            "fp64": {"value": nobs / (ms64 * 1e-3), "unit": UNIT, "ms_per_step": ms64},
            "plain": {"value": 1.0 / (ms1 * 1e-3), "unit": UNIT, "path": "nsg_exp_value, one observable per call"},
            "mixed_rel_err_vs_fp64": {"max": float(err.max()), "median": float(np.median(err)),
                                      "per_observable": [float(x) for x in err]},
            # per call: Pauli frames, the pair launch, the two reduction passes (frames and tables are cached)
            "clocks": clocks.summary(), "gpu_launches": 4 * args.steps}
    print(json.dumps(line))


def run_batch512(args, torch, L):
    """512 circuits, n ~ U[8, 64], t ~ U[4, 32], 20·n Clifford gates, 16 dense
    Paulis each: every ⟨P⟩ of every circuit in one persistent launch per row
    width (nsg_exp_value_multi), against the plain path run per circuit and
    per observable (nsg_exp_value)."""
    from stab_decomp_simulator_rust_gb300 import (PRECISION_FP64, PRECISION_MIXED, BatchPlan, PauliString,
                                                  QuantumState, exp_values_multi)
    from stab_decomp_simulator_rust_gb300 import workloads as W
    circuits = W.batch_circuits()
    stream = torch.cuda.current_stream()
    pinned = [torch.from_numpy(np.ascontiguousarray(g)).pin_memory().numpy() for _, g, _ in circuits]
    t0 = time.perf_counter()
    states = [QuantumState.from_gates(n, g) for (n, _, _), g in zip(circuits, pinned)]
    compile_s = time.perf_counter() - t0
    for s in states:
        s.set_stream(stream.cuda_stream)
    plists = [[PauliString.dense(p) for p in ps] for _, _, ps in circuits]
    chis = [s.stabilizer_rank for s in states]
    pairs = sum(c * (c + 1) // 2 for c in chis)
    nobs = sum(len(p) for p in plists)
    # the batched path as a captured plan (CUDA graph; kernel variant tuned on a sample at creation)
    t0 = time.perf_counter()
    plan = BatchPlan(states, plists, PRECISION_MIXED)
    plan_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        plan.run()
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    msmx, vmx = _timed(torch, stream, plan.run, args.steps)
    msdir, _ = _timed(torch, stream, lambda: exp_values_multi(states, plists, PRECISION_MIXED), 1)
    ms64, v64 = _timed(torch, stream, lambda: exp_values_multi(states, plists, PRECISION_FP64), args.steps)
    # plain: one circuit and one observable per call, FP64
    npl = min(args.plain_circuits, len(states))

    def plain():
        return [[states[c].exp_value(p) for p in plists[c]] for c in range(npl)]
    mspl, vpl = _timed(torch, stream, plain, 1)
    # the batched mixed path (captured plan) on the same circuits, for a like-for-like ratio
    sub = BatchPlan(states[:npl], plists[:npl], PRECISION_MIXED)
    sub.run()
    mssub, _ = _timed(torch, stream, sub.run, 1)
    clocks.stop()
    obs_pl = sum(len(plists[c]) for c in range(npl))
    err = np.concatenate([_rel_err(a, b) for a, b in zip(vmx, v64)])
    err_pl = np.concatenate([_rel_err(np.asarray(vpl[c]), v64[c]) for c in range(npl)])
    # end to end: compile from pinned host gate lists + the batched call
    t0 = time.perf_counter()
    st2 = [QuantumState.from_gates(n, g) for (n, _, _), g in zip(circuits, pinned)]
    exp_values_multi(st2, plists, PRECISION_MIXED)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    del st2
    line = {"metric": METRIC, "value": nobs / (msmx * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": msmx, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 accumulation of exact pair values, f64 final reduction",
            "data": "synthetic (seeded generator)",
            "config": {"workload": "512 circuits, n~U[8,64], t~U[4,32], 20n {H,S,CX}, 16 dense Paulis each (seed 4)",
                       "chi_min": min(chis), "chi_max": max(chis), "chi_sum": sum(chis), "pairs_total": pairs,
                       "observables": nobs, "l2": "inputs larger than L2 (term tables of 512 states)",
                       "compile_s_all_circuits": compile_s},
            "inner_products_per_s": sum(c * (c + 1) // 2 * len(p) for c, p in zip(chis, plists)) / (msmx * 1e-3),
            "plan": {"create_s": plan_s, "tiling": plan.tiling,
                     "path": "nsg_plan_run: CUDA-graph replay of frames, term tables, Pauli frames, pair launches, "
                             "reductions and the result copy"},
            "direct_batched_mixed": {"value": nobs / (msdir * 1e-3), "unit": UNIT, "ms": msdir,
                                     "path": "nsg_exp_value_multi"},
            "fp64_batched": {"value": nobs / (ms64 * 1e-3), "unit": UNIT, "ms_per_step": ms64},
            "plain": {"value": obs_pl / (mspl * 1e-3), "unit": UNIT, "circuits": npl, "ms": mspl,
                      "path": "nsg_exp_value per circuit and observable, FP64"},
            "speedup_mixed_batched_vs_plain_same_circuits": mspl / mssub,
            "rel_err": {"mixed_vs_fp64_batched_max": float(err.max()), "plain_vs_fp64_batched_max": float(err_pl.max())},
            "e2e": {"value": nobs / e2e_s, "unit": UNIT, "s": e2e_s,
                    "h2d_bytes_per_step": int(sum(g.nbytes for g in pinned) + sum(p.ops.nbytes for ps in plists for p in ps)),
                    "d2h_bytes_per_step": int(8 * nobs),
                    "path": "nsg_state_from_circuit x512 + nsg_exp_value_multi, host buffers"},
            "clocks": clocks.summary(),
            # per replay: frames and term tables per state, Pauli frames per state, and per row width
            # (32- and 64-bit) one pair launch and two reduction passes
            "gpu_launches": args.steps * (3 * len(states) + 3 * len({n <= 32 for (n, _, _) in circuits}))}
    print(json.dumps(line))


def run_project64(args, torch, L):
    """n=64, 8000 {H,S,CX} + 40 T: project qubits 0-7 onto seeded outcomes
    (the last projection renormalises in FP64), then 10^6 samples of qubits
    8-15.  The samples come from one pass over the 256 Z-strings on 8-15; the
    same pass in mixed precision is compared with FP64, and the sample
    histogram with the FP64 marginal (total-variation distance)."""
    from stab_decomp_simulator_rust_gb300 import PRECISION_FP64, PRECISION_MIXED, PauliString, QuantumState
    from stab_decomp_simulator_rust_gb300 import workloads as W
    cfg = W.PROJECT_N64
    n = cfg["n"]
    gates = W.random_clifford_t_circuit(n, cfg["num_clifford"], cfg["num_t"], cfg["seed"])
    rng = W.Xoshiro256ss(cfg["seed"] + 200)
    outcomes = [rng.below(2) for _ in range(cfg["num_project"])]
    stream = torch.cuda.current_stream()
    clocks = ClockSampler(0)
    clocks.start()
    t0 = time.perf_counter()
    st = QuantumState.from_gates(n, gates)
    torch.cuda.synchronize()
    compile_s = time.perf_counter() - t0
    st.set_stream(stream.cuda_stream)
    chi0 = st.stabilizer_rank

    def project():
        for q, o in enumerate(outcomes[:-1]):
            st.project_unnormalized(q, bool(o))
        st.project_normalized(len(outcomes) - 1, bool(outcomes[-1]))
    ms_proj, _ = _timed(torch, stream, project, 1)
    chi1 = st.stabilizer_rank
    ms_norm, norm = _timed(torch, stream, st.norm, 1)
    qargs = list(range(8, 16))
    zs = []
    for S in range(256):
        ops = np.zeros(n, np.uint8)
        for i in range(8):
            if (S >> i) & 1:
                ops[qargs[i]] = 3
        zs.append(PauliString.dense(ops))
    ms_mx, e_mx = _timed(torch, stream, lambda: st.exp_values(zs, PRECISION_MIXED), 1)
    ms_64, e_64 = _timed(torch, stream, lambda: st.exp_values(zs, PRECISION_FP64), 1)

    def marginal(e):
        e = np.asarray(e, float).copy()
        h = 1
        while h < 256:
            for i in range(0, 256, 2 * h):
                a, b = e[i:i + h].copy(), e[i + h:i + 2 * h].copy()
                e[i:i + h], e[i + h:i + 2 * h] = a + b, a - b
            h *= 2
        return np.maximum(e / (256.0 * e_64[0]), 0.0)
    p64, pmx = marginal(e_64), marginal(e_mx)
    shots = cfg["shots"]
    ms_samp, (vals, cnts) = _timed(torch, stream, lambda: st.sample_raw(qargs, shots, seed=cfg["seed"]), 1)
    clocks.stop()
    hist = np.zeros(256)
    for v, c in zip(vals, cnts):
        hist[v] += c
    tvd = 0.5 * float(np.abs(hist / shots - p64).sum())
    line = {"metric": METRIC, "value": 256 / (ms_mx * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": 1,
            "warmup": 0, "ms_per_step": ms_mx, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 accumulation of exact pair values, f64 final reduction", "data": "synthetic (seeded generator)",
            "config": {"workload": "n=64, 8000 {H,S,CX} + 40 T (seed 5); project q0-7 onto seeded outcomes; "
                                   "1e6 samples of q8-15", "outcomes_q0_7": outcomes, "chi_compiled": chi0,
                       "chi_after_projection": chi1, "pairs_per_observable": chi1 * (chi1 + 1) // 2,
                       "compile_s": compile_s, "l2": "inputs larger than L2"},
            "stage_ms": {"project_and_renormalise": ms_proj, "norm_fp64": ms_norm,
                         "z_strings_256_mixed": ms_mx, "z_strings_256_fp64": ms_64, "sample_1e6": ms_samp},
            "norm_after_renormalise": norm, "norm_error": abs(norm - 1.0),
            "marginal_max_abs_diff_mixed_vs_fp64": float(np.abs(pmx - p64).max()),
            "tvd_samples_vs_fp64_marginal": tvd,
            "tvd_expected_from_sampling_noise": 0.5 * float(np.sqrt(2.0 * p64 * (1 - p64) / (np.pi * shots)).sum()),
            "clocks": clocks.summary()}
    print(json.dumps(line))


def run_workload(args):
    torch, L = _setup_gpu()
    {"precision60": run_precision60, "batch512": run_batch512,
     "project64": run_project64}[args.workload](args, torch, L)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--workload", default="plain40", choices=["plain40", "precision60", "batch512", "project64"],
                    help="plain40: the headline line; the others measure the precision, batching and "
                         "projection/sampling workloads (one JSON line each)")
    ap.add_argument("--plain-circuits", type=int, default=512,
                    help="batch512: circuits timed on the plain per-circuit path")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "plain40":
        run_ours(args)
    else:
        run_workload(args)


if __name__ == "__main__":
    main()
