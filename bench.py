"""Benchmark: Pauli expectation values per second, mixed+batched vs plain FP64.

Default workload (the batching form the metric's ≥10× target is quoted on):
512 independent circuits, n ~ U[8, 64], t ~ U[4, 32], 20·n random
{H, S, CX} gates each (seeded per circuit, stab_decomp_simulator_rust_gb300/
workloads.py), 16 random dense Pauli observables per circuit: 8,192 ⟨P⟩ per
step over Σχ(χ+1)/2 ≈ 1.04·10⁹ term pairs.

* ``value``: ⟨P⟩/s of the batched mixed-precision path with the 512 compiled
  states resident in HBM: every ⟨P⟩ of every circuit in one captured plan
  (nsg_plan_run: one CUDA-graph replay per step — frames, term tables, Pauli
  frames, one persistent pair launch per row width, the reductions and the
  copy of 8,192 doubles to pinned host memory), timed with CUDA events on
  the stream the states run on.  The term tables of the 512 states (≈ 3 GB)
  are larger than L2.
* ``plain``: the drop-in single-observable FP64 path (nsg_exp_value, one
  circuit and one observable per call) on the same circuits;
  ``speedup_vs_plain`` = value ÷ plain.
* ``exactness``: every one of the 8,192 results of the timed path (and of
  the FP64 batched path) against the exact sum of its pair terms
  (nsg_exp_value_counts: integer counts per power of √2, evaluated exactly).
* ``zero_screen``: the common-stabilizer test (nsg_zero_screen, host work,
  not used by ``value``): how many of the exactly-zero observables it decides
  without pair work, and how many it decides that are not zero (must be 0).
* ``screened``: an opt-in use of that test, not the metric: the states whose
  every observable it decides are not summed (their results are the exact
  0); one captured plan over the other states plus the host test per step,
  with every result checked against the exact sums.
* ``e2e``: the same metric end to end through the C ABI from host buffers:
  nsg_states_from_circuits (512 gate lists from pinned host memory) +
  nsg_exp_value_multi (Paulis from host, 8,192 doubles back), wall clock.
* ``roofline``: the pair kernel (integer pipe) — w·w·W 64-bit word
  operations per pair (w = the circuit's n) ÷ its event-timed launches,
  against the measured integer-logic peak of the same GPU.
* ``gate_apply``: Clifford application on HBM-resident terms (n = 60,
  χ = 26,244 and n = 64, χ = 78,732): per-gate algorithmic bytes ÷ time,
  fused (one launch for 1,000 gates) and gate by gate (one launch per gate).
* ``plain40``: the n = 40 plain-method workload (4000 + 24 T, χ = 972,
  64 dense Paulis) as a second line item.
* ``cpu_baseline`` / ``--impl reference``: the C++ restatement of the
  reference's Rust path (the reference cannot be built here: no Rust
  toolchain) on the host cores: per step one circuit drawn from the 512 in
  proportion to its expected cost, compiled with the reference's compile loop
  and timed on a uniform sample of its term pairs; the whole workload's time
  is the Horvitz-Thompson estimate over the steps.

Other workloads (one JSON line each): --workload plain40 | precision60 |
project64 | gates.

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

METRIC = "Pauli ⟨P⟩/s and CH inner products/s, mixed+batched vs plain FP64 @≤1e-9 err"
UNIT = "<P>/s"
WORKLOAD = "512 circuits, n~U[8,64], t~U[4,32], 20n {H,S,CX}, 16 dense Paulis each (seed 4)"

# DRAM bytes (read + write) of the 64-bit-row pair launch of one step of the
# default workload, with the tiling its plan tunes (16 kets per chunk, 256
# tasks per resident warp), from one ncu capture of that launch:
# dram__bytes_read.sum 3.31 GB + dram__bytes_write.sum 0.48 GB (the ket
# tables ≈ 2 GB read about once, task records, frames).  The kernel's later
# arithmetic changes left its reads unchanged (296 MB on a 20-state capture
# before and after them).
PAIR_TRAFFIC_BYTES = 3_310_000_000 + 483_440_000


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
# The reference's CPU path on the host cores (the oracle port of it)
def oracle_batch_estimate(circuits, steps: int, step_pair_seconds: float, threads: int, seed: int = 11,
                          single_thread: bool = False):
    """Times the reference algorithm on the batching workload, one sampled circuit per step.

    Step k draws circuit c with probability q_c ∝ P_c·n_c³ (P_c: the pair
    count of its T-expansion size, an upper bound of its compiled pair count;
    the reference's per-pair cost grows about as n³), compiles it with the
    reference's compile loop on all `threads`, and times a uniform sample of
    its term pairs (one of its observables, the reference inner-product
    algorithm) for about `step_pair_seconds`.  The workload's time is the
    Horvitz-Thompson estimate mean_k[(compile_k + 16·pairs_k·sec_per_pair_k)
    / q_k]: draws in proportion to the expected cost keep its spread small,
    since the pair evaluations are nearly all of the time."""
    from oracle import pyoracle as po
    N = len(circuits)
    nobs = sum(len(ps) for _, _, ps in circuits)
    tcount = [int((np.asarray(g)[:, 0] == 11).sum() + (np.asarray(g)[:, 0] == 12).sum()) for _, g, _ in circuits]
    chiT = np.asarray([po.t_tensor_rank(t) if t else 1 for t in tcount], dtype=np.float64)
    P = chiT * (chiT + 1) / 2
    nq = np.asarray([n for n, _, _ in circuits], dtype=np.float64)
    q = P * nq ** 3 / (P * nq ** 3).sum()
    rng = np.random.default_rng(seed)
    est, step_ms, draws = [], [], []
    last = None
    for k in range(steps):
        t_step = time.perf_counter()
        c = int(rng.choice(N, p=q))
        n, gates, ops = circuits[c]
        t0 = time.perf_counter()
        st, _ = po.OracleState.compile_terms(n, gates, np.arange(int(chiT[c]), dtype=np.int64), threads)
        comp = time.perf_counter() - t0
        chi = st.stabilizer_rank
        pairs = chi * (chi + 1) // 2
        o = ops[k % len(ops)]
        sec, _ = st.time_pairs(0, o, None, 64 * threads, 1 + k, threads)  # calibration
        npairs = int(max(64 * threads, min(4 * pairs + 1000, step_pair_seconds * 64 * threads / max(sec, 1e-9))))
        sec, _ = st.time_pairs(0, o, None, npairs, 100 + k, threads)
        spp = sec / npairs
        est.append((comp + len(ops) * pairs * spp) / q[c])
        step_ms.append(1e3 * (time.perf_counter() - t_step))
        draws.append({"circuit": c, "n": n, "chi": chi, "compile_s": comp, "pairs_timed": npairs,
                      "pairs_per_s": npairs / sec})
        last = (st, o, npairs / sec)
    total_s = float(np.mean(est))
    stderr_s = float(np.std(est, ddof=1) / np.sqrt(len(est))) if len(est) > 1 else None
    out = {"value": nobs / total_s, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": (f"{steps} circuits drawn from the 512 in proportion to pairs x n^3 (their expected cost); each "
                      f"compiled with the reference compile loop on {threads} threads and timed on a uniform sample "
                      f"of ~{step_pair_seconds:.1f} s of its term pairs (reference inner-product algorithm); the "
                      f"{nobs} <P> of all 512 circuits extrapolated by the Horvitz-Thompson estimate"),
           "workload_seconds_estimate": total_s, "workload_seconds_stderr": stderr_s,
           "step_ms": step_ms, "draws": draws}
    if single_thread and last is not None:
        st, o, rate_all = last
        n1 = max(200, int(rate_all / threads))
        sec1, _ = st.time_pairs(0, o, None, n1, 999, 1)
        ratio = (n1 / sec1) / rate_all
        out["single_thread"] = {"value": out["value"] * ratio, "unit": UNIT, "cores": 1,
                                "note": "the reference's own threading (one thread): the estimate scaled by the "
                                        "measured 1-thread / all-thread pair rate on the last drawn circuit",
                                "pair_rate_ratio": ratio}
    return out


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from stab_decomp_simulator_rust_gb300 import workloads as W
    circuits = W.batch_circuits()
    threads = os.cpu_count() or 1
    # warm-up: the first draw's compile and a short pair sample (page-in of the library and the data)
    oracle_batch_estimate(circuits, max(0, min(args.warmup, 1)), 0.2, threads, seed=1)
    r = oracle_batch_estimate(circuits, args.steps, args.ref_step_seconds, threads, seed=11, single_thread=True)
    ms = statistics.mean(r["step_ms"])
    line = {"impl": "reference", "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
            "config": {"workload": WORKLOAD, "parallelism": "host threads"},
            "cpu_baseline": {k: r[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": r["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "single_thread": r.get("single_thread"),
            "estimate": {"workload_seconds": r["workload_seconds_estimate"],
                         "stderr_seconds": r["workload_seconds_stderr"], "draws": r["draws"]}}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
def _setup_gpu(local=0):
    import torch
    from stab_decomp_simulator_rust_gb300 import _ffi, build
    torch.cuda.set_device(local)
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
    return tot / max(steps, 1), out


def _int_peak(L):
    """Measured integer-logic peak: 64-bit word operations per second (2 LOP3 per word)."""
    import ctypes as C
    from stab_decomp_simulator_rust_gb300 import _ffi
    probe_s, probe_ops = C.c_double(), C.c_uint64()
    _ffi.check(L.nsg_probe_int_ops(20000, C.byref(probe_s), C.byref(probe_ops)))
    return probe_ops.value / probe_s.value / 2.0


def _pair_profile(L, fn):
    """Runs fn() with pair-kernel profiling on: (ms summed over launches, launches, pairs)."""
    import ctypes as C
    from stab_decomp_simulator_rust_gb300 import _ffi
    _ffi.check(L.nsg_profile_enable(1))
    _ffi.check(L.nsg_profile_read(None, None, None))
    fn()
    ms, nl, pr = C.c_double(), C.c_uint64(), C.c_uint64()
    _ffi.check(L.nsg_profile_read(C.byref(ms), C.byref(nl), C.byref(pr)))
    _ffi.check(L.nsg_profile_enable(0))
    return ms.value, nl.value, pr.value


def _exact_errors(vals, exact):
    vals, exact = np.asarray(vals, float), np.asarray(exact, float)
    d = np.abs(vals - exact)
    nz = exact != 0
    rel = d[nz] / np.abs(exact[nz])
    return {"max_abs_err": float(d.max()) if len(d) else 0.0,
            "max_rel_err_nonzero": float(rel.max()) if len(rel) else 0.0,
            "median_rel_err_nonzero": float(np.median(rel)) if len(rel) else 0.0,
            "exact_zero_observables": int((~nz).sum()),
            "max_abs_err_on_exact_zeros": float(d[~nz].max()) if (~nz).any() else 0.0,
            "observables": int(len(d))}


def _gate_bytes(op, w):
    """Algorithmic bytes per (gate, term) of the packed layout (W = 1 word per row):
    S 3·8W+2, CX 9·8W+3, H 5·8W + 2·(3·w·8W) (prepare step + the column
    operations of the resolve, one full G/F/M read and write)."""
    W = (w + 63) // 64
    return {0: 5 * 8 * W + 2 * 3 * w * 8 * W, 4: 3 * 8 * W + 2, 8: 9 * 8 * W + 3}[int(op)]


def gate_apply_leg(torch, stream, hbm_gbs):
    """Clifford application (nsg_apply_gates) on HBM-resident terms of the
    n = 60 and n = 64 workloads: 1,000 random {H,S,CX} gates fused in one
    launch, and 48 of them gate by gate (one call each), also split by kind."""
    from stab_decomp_simulator_rust_gb300 import QuantumState
    from stab_decomp_simulator_rust_gb300 import workloads as W
    out = {}
    for name, cfg in (("n60_chi26244", W.PRECISION_N60), ("n64_chi78732", W.PROJECT_N64)):
        n = cfg["n"]
        st = QuantumState.from_gates(n, W.random_clifford_t_circuit(n, cfg["num_clifford"], cfg["num_t"], cfg["seed"]))
        st.set_stream(stream.cuda_stream)
        chi = st.stabilizer_rank
        run = W.random_clifford_t_circuit(n, 1000, 0, cfg["seed"] + 300)
        bytes_run = sum(_gate_bytes(g[0], n) for g in run) * chi
        st.apply_gates(run[:10])
        ms_fused, _ = _timed(torch, stream, lambda: st.apply_gates(run), 3)
        one = run[:48]
        bytes_one = sum(_gate_bytes(g[0], n) for g in one) * chi
        ms_one, _ = _timed(torch, stream, lambda: [st.apply_gates(one[i:i + 1]) for i in range(len(one))], 2)
        term_bytes = 2 * (3 * 64 * 8 + 4 * 8 + 6)  # one read and one write of a whole term (n ≤ 64)
        # by kind: H moves every term through a warp; S and CX (row kernel) touch their rows only
        h_one = one[one[:, 0] == 0]
        r_one = one[one[:, 0] != 0]
        ms_h, _ = _timed(torch, stream, lambda: [st.apply_gates(h_one[i:i + 1]) for i in range(len(h_one))], 2)
        ms_r, _ = _timed(torch, stream, lambda: [st.apply_gates(r_one[i:i + 1]) for i in range(len(r_one))], 2)
        bytes_r = sum(_gate_bytes(g[0], n) for g in r_one) * chi
        out[name] = {
            "chi": chi, "state_bytes": int(chi * term_bytes // 2),
            "fused_1000_gates": {"ms": ms_fused, "algorithmic_GBps": bytes_run / (ms_fused * 1e-3) / 1e9,
                                 "frac_of_hbm": bytes_run / (ms_fused * 1e-3) / 1e9 / hbm_gbs,
                                 "term_traffic_GBps": chi * term_bytes / (ms_fused * 1e-3) / 1e9},
            "gate_by_gate": {"ms_per_gate": ms_one / len(one),
                             "algorithmic_GBps": bytes_one / (ms_one * 1e-3) / 1e9,
                             "frac_of_hbm": bytes_one / (ms_one * 1e-3) / 1e9 / hbm_gbs,
                             "h_gates": {"count": len(h_one), "ms_per_gate": ms_h / max(len(h_one), 1),
                                         "term_traffic_GBps": len(h_one) * chi * term_bytes / (ms_h * 1e-3) / 1e9,
                                         "term_traffic_frac_of_hbm":
                                             len(h_one) * chi * term_bytes / (ms_h * 1e-3) / 1e9 / hbm_gbs},
                             "s_cx_gates": {"count": len(r_one), "ms_per_gate": ms_r / max(len(r_one), 1),
                                            "algorithmic_GBps": bytes_r / (ms_r * 1e-3) / 1e9,
                                            "frac_of_hbm": bytes_r / (ms_r * 1e-3) / 1e9 / hbm_gbs}}}
        del st
    out["hbm_peak_GBps"] = hbm_gbs
    out["note"] = ("algorithmic bytes per (gate, term): S 3*8W+2, CX 9*8W+3, H 5*8W+2*(3*w*8W); a launch with H "
                   "holds whole terms in registers (one read and write of every term whatever its gates); a call "
                   "with a single S or CX updates only the rows it touches (one thread per term)")
    return out


def plain40_leg(torch, stream, L, steps, warmup):
    """The n = 40 plain-method workload: 64 ⟨P⟩ as a captured FP64 plan (device-resident), the
    drop-in single-observable path, and end to end from host buffers."""
    from stab_decomp_simulator_rust_gb300 import PRECISION_FP64, BatchPlan, PauliString, QuantumState
    from stab_decomp_simulator_rust_gb300 import workloads as W
    cfg = W.PLAIN_N40
    n = cfg["n"]
    gates = W.random_clifford_t_circuit(n, cfg["num_clifford"], cfg["num_t"], cfg["seed"])
    paulis = [PauliString.dense(p) for p in W.random_dense_paulis(n, cfg["num_paulis"], cfg["seed"] + 100)]
    st = QuantumState.from_gates(n, gates)
    st.set_stream(stream.cuda_stream)
    chi = st.stabilizer_rank
    plan = BatchPlan([st], [paulis], PRECISION_FP64)
    for _ in range(warmup):
        plan.run()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    tot = 0.0
    for _ in range(steps):
        flush.zero_()
        ms, _ = _timed(torch, stream, plan.run, 1)
        tot += ms
    ms_plan = tot / steps
    st.exp_value(paulis[0])
    ms_plain, _ = _timed(torch, stream, lambda: [st.exp_value(p) for p in paulis[:8]], 1)
    pinned = torch.from_numpy(np.ascontiguousarray(gates)).pin_memory().numpy()
    QuantumState.from_gates(n, pinned).exp_values(paulis)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        s2 = QuantumState.from_gates(n, pinned)
        s2.exp_values(paulis)
        del s2
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / steps
    return {"workload": "n=40, 4000 {H,S,CX} + 24 T (seed 2), 64 dense Paulis (seed 102)", "chi": chi,
            "value": len(paulis) / (ms_plan * 1e-3), "unit": UNIT, "ms_per_step": ms_plan,
            "path": "BatchPlan.run (CUDA-graph replay), FP64; L2 flushed before every step",
            "plain": {"value": 8 / (ms_plain * 1e-3), "unit": UNIT, "path": "nsg_exp_value, one observable per call"},
            "e2e": {"value": len(paulis) / (e2e_ms * 1e-3), "unit": UNIT, "ms_per_step": e2e_ms,
                    "path": "nsg_state_from_circuit + nsg_exp_value_batch, host buffers"}}


def run_ours(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch, L = _setup_gpu(local)
    from stab_decomp_simulator_rust_gb300 import (PRECISION_FP64, PRECISION_MIXED, BatchPlan, PauliString,
                                                  QuantumState, exp_values_multi)
    from stab_decomp_simulator_rust_gb300 import workloads as W
    from stab_decomp_simulator_rust_gb300.state import counts_to_value

    circuits = W.batch_circuits()
    stream = torch.cuda.current_stream()
    pinned = [torch.from_numpy(np.ascontiguousarray(g)).pin_memory().numpy() for _, g, _ in circuits]
    plists = [[PauliString.dense(p) for p in ps] for _, _, ps in circuits]
    nobs = sum(len(p) for p in plists)
    t0 = time.perf_counter()
    states = QuantumState.from_gates_many([(n, g) for (n, _, _), g in zip(circuits, pinned)])
    torch.cuda.synchronize()
    compile_s = time.perf_counter() - t0
    for s in states:
        s.set_stream(stream.cuda_stream)
    chis = [s.stabilizer_rank for s in states]
    ns = [n for n, _, _ in circuits]
    pairs = [c * (c + 1) // 2 for c in chis]

    # ---- the timed path: the mixed+batched captured plan
    t0 = time.perf_counter()
    plan = BatchPlan(states, plists, PRECISION_MIXED)
    plan_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        plan.run()
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    ms_step, vmx = _timed(torch, stream, plan.run, args.steps)
    torch.cuda.synchronize()
    clocks.stop()
    ms_step, value = combine_ranks(ms_step, nobs, "cuda")

    # ---- FP64 batched (captured plan) and the exact sums of every observable
    plan64 = BatchPlan(states, plists, PRECISION_FP64)
    plan64.run()
    ms64, v64 = _timed(torch, stream, plan64.run, max(1, min(3, args.steps)))
    del plan64
    t0 = time.perf_counter()
    exact = []
    for s, ps in zip(states, plists):
        counts, scale = s.exp_value_counts(ps)
        exact.append([counts_to_value(c, scale=scale) for c in counts])
    exact_s = time.perf_counter() - t0
    flat = lambda xs: np.concatenate([np.asarray(x, float) for x in xs])
    exactness = {"mixed_batched_vs_exact": _exact_errors(flat(vmx), flat(exact)),
                 "fp64_batched_vs_exact": _exact_errors(flat(v64), flat(exact)),
                 "exact_path": "nsg_exp_value_counts per circuit (signed counts per power of sqrt 2), summed exactly",
                 "exact_s": exact_s}
    # ---- the common-stabilizer zero test (host only, not used by the timed path): how many of the
    # exactly-zero observables it decides without pair work, and that every one it decides is zero
    t0 = time.perf_counter()
    screened = np.concatenate([s.zero_screen(ps) for s, ps in zip(states, plists)])
    screen_s = time.perf_counter() - t0
    ex_flat = flat(exact)
    zero_screen = {"decided_zero": int(screened.sum()), "exact_zero": int((ex_flat == 0.0).sum()),
                   "decided_but_nonzero": int((screened & (ex_flat != 0.0)).sum()), "observables": int(len(ex_flat)),
                   "host_s": screen_s,
                   "note": "nsg_zero_screen: P anticommutes with a stabilizer common to every term; not used by value"}
    # Opt-in use of the test (not the metric): states whose every observable it decides are not summed;
    # one captured plan over the others, plus the host test of all 512 states, per step.
    per_state = [s.zero_screen(ps) for s, ps in zip(states, plists)]
    rest = [i for i, z in enumerate(per_state) if not z.all()]
    screened_line = None
    if rest:
        splan = BatchPlan([states[i] for i in rest], [plists[i] for i in rest], PRECISION_MIXED)
        vs = splan.run()
        ms_s, _ = _timed(torch, stream, splan.run, max(1, min(3, args.steps)))
        del splan
        got = [np.zeros(len(ps)) for ps in plists]
        for k, i in enumerate(rest):
            got[i] = np.asarray(vs[k], float)
        ms_tot = ms_s + 1e3 * screen_s
        screened_line = {"value": nobs / (ms_tot * 1e-3), "unit": UNIT, "ms_per_step": ms_tot,
                         "states_not_summed": len(states) - len(rest), "vs_exact": _exact_errors(flat(got), ex_flat),
                         "note": "opt-in: the states whose observables nsg_zero_screen decides are not summed "
                                 "(their results are the exact 0); one plan over the other states + the host "
                                 "test per step; not the metric"}

    # ---- plain: one circuit and one observable per call, FP64 (4 of the 16 observables of every circuit)
    per = max(1, min(args.plain_observables, 16))
    for s, ps in zip(states, plists):  # bra frames and term tables of every state are cached by now
        s.exp_value(ps[0])
    ms_plain, vpl = _timed(torch, stream, lambda: [[s.exp_value(p) for p in ps[:per]] for s, ps in zip(states, plists)], 1)
    plain_value = per * len(states) / (ms_plain * 1e-3)
    plain_err = _exact_errors(flat(vpl), flat([e[:per] for e in exact]))

    # ---- roofline of the pair kernel: the direct batched call with its launches event-timed
    pk_ms, pk_launches, pk_pairs = _pair_profile(L, lambda: exp_values_multi(states, plists, PRECISION_MIXED))
    ops = float(sum(p * n * n for p, n in zip(pairs, ns)))  # w·w·W per pair, W = 1 (n ≤ 64)
    word_peak = _int_peak(L)
    achieved = ops / (pk_ms * 1e-3)
    roofline = {"bound": "int", "achieved": achieved / 1e12, "peak": word_peak / 1e12, "unit": "Tword-ops/s",
                "frac": achieved / word_peak, "traffic": PAIR_TRAFFIC_BYTES,
                "traffic_unit": "DRAM bytes of the 64-bit-row launch of one step (ncu, tuned tiling); "
                                "the ket tables it reads are ~2.0 GB",
                "kernel": "pair_kernel (32- and 64-bit-row launches of one step)",
                "peak_source": "measured on this GPU: LOP3 chains on every SM (nsg_probe_int_ops), "
                               "a 64-bit word = 2 int32 logic ops",
                "algorithmic_unit": "n*n 64-bit word-ops per term pair (w*w*W, W=1), summed over the 512 circuits",
                "pair_kernel_ms_per_step": pk_ms, "launches_per_step": pk_launches, "pairs_per_step": pk_pairs}

    # ---- end to end from host buffers
    e2e_steps = max(1, min(3, args.steps))
    src = [(n, g) for (n, _, _), g in zip(circuits, pinned)]
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        st2 = QuantumState.from_gates_many(src)
        exp_values_multi(st2, plists, PRECISION_MIXED)
        del st2
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / e2e_steps
    e2e = {"value": ws * nobs / (e2e_ms * 1e-3), "unit": UNIT, "ms_per_step": e2e_ms,
           "h2d_bytes_per_step": int(sum(g.nbytes for g in pinned) + sum(p.ops.nbytes for ps in plists for p in ps)
                                     + 24 * nobs),
           "d2h_bytes_per_step": int(8 * nobs),
           "path": "nsg_states_from_circuits (512 circuits) + nsg_exp_value_multi (mixed), host buffers; "
                   "states freed inside the step"}

    hbm = None
    try:
        hbm = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
    except Exception:
        hbm = 6800.0
    gates_leg = gate_apply_leg(torch, stream, hbm) if not args.no_gates else None
    p40 = plain40_leg(torch, stream, L, max(3, min(args.steps, 10)), 3) if not args.no_plain40 else None

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 accumulation of exact pair values, f64 final reduction",
            "data": "synthetic (seeded generator)",
            "config": {"workload": WORKLOAD, "chi_min": min(chis), "chi_max": max(chis), "chi_sum": sum(chis),
                       "pairs_per_step": int(sum(pairs)), "observables_per_step": nobs,
                       "l2": "inputs larger than L2 (term tables of 512 states)", "parallelism": f"replicas x{ws}"},
            "inner_products_per_s": sum(p * len(ps) for p, ps in zip(pairs, plists)) / (ms_step * 1e-3),
            "path": "BatchPlan.run (nsg_plan_run: CUDA-graph replay), mixed precision",
            "plan": {"create_s": plan_s, "tiling": plan.tiling},
            "compile_s_512_circuits": compile_s,
            "fp64_batched": {"value": nobs / (ms64 * 1e-3), "unit": UNIT, "ms_per_step": ms64},
            "plain": {"value": plain_value, "unit": UNIT, "ms": ms_plain, "observables": per * len(states),
                      "path": f"nsg_exp_value, one circuit and one observable per call, FP64 "
                              f"({per} of the 16 observables of each of the 512 circuits)",
                      "vs_exact": plain_err},
            "speedup_vs_plain": value / plain_value,
            "exactness": exactness, "zero_screen": zero_screen, "screened": screened_line, "e2e": e2e, "roofline": roofline, "gate_apply": gates_leg,
            "plain40": p40, "clocks": clocks.summary(),
            # per replay: frames and term tables per state, Pauli frames per state, and per row
            # width (32- and 64-bit) one pair launch and two reduction passes
            "gpu_launches": args.steps * (3 * len(states) + 3 * len({n <= 32 for n in ns}))}
    if rank == 0:
        if not args.no_cpu:
            try:
                r = oracle_batch_estimate(circuits, args.cpu_steps, 1.0, os.cpu_count() or 1, seed=21)
                line["cpu_baseline"] = {k: r[k] for k in ("value", "unit", "cores", "kind", "sample")}
            except Exception as e:  # the oracle is optional for the GPU number itself
                line["cpu_baseline"] = {"value": None, "error": str(e)}
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()


# ---------------------------------------------------------------------------
# The other workloads (one JSON line each)
def run_precision60(args, torch, L):
    """n=60, 6000 {H,S,CX} + 36 T, 256 sparse Paulis of weight 1..8: FP64 and
    mixed accumulation over the full χ² pair sum; per-observable error of both
    against the exact sum of every pair term."""
    from stab_decomp_simulator_rust_gb300 import PRECISION_FP64, PRECISION_MIXED, PauliString, QuantumState
    from stab_decomp_simulator_rust_gb300 import workloads as W
    from stab_decomp_simulator_rust_gb300.state import counts_to_value
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
    t0 = time.perf_counter()
    counts, scale = st.exp_value_counts(paulis)
    ms_exact = (time.perf_counter() - t0) * 1e3
    exact = np.asarray([counts_to_value(c, scale=scale) for c in counts])
    nobs = len(paulis)

    def per_obs(v):
        v = np.asarray(v, float)
        d = np.abs(v - exact)
        return [float(x) for x in np.where(exact != 0, d / np.maximum(np.abs(exact), 1e-300), d)]
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
            "exact": {"ms": ms_exact, "path": "nsg_exp_value_counts: signed counts per power of sqrt 2, summed exactly"},
            "mixed_vs_exact": _exact_errors(vmx, exact), "fp64_vs_exact": _exact_errors(v64, exact),
            "per_observable_err_vs_exact": {"note": "relative where the exact value is nonzero, else absolute",
                                            "mixed": per_obs(vmx), "fp64": per_obs(v64)},
            "clocks": clocks.summary(), "gpu_launches": 4 * args.steps}
    print(json.dumps(line))


def run_project64(args, torch, L):
    """n=64, 8000 {H,S,CX} + 40 T: project qubits 0-7 onto seeded outcomes
    (the last projection renormalises in FP64), then 10^6 samples of qubits
    8-15.  The samples come from one pass over the 256 Z-strings on 8-15; the
    marginal is also computed exactly (exact counts of every pair term of the
    256 Z-strings, Walsh transform in exact arithmetic), and the sample
    histogram is compared with it (total-variation distance)."""
    from fractions import Fraction

    from stab_decomp_simulator_rust_gb300 import PRECISION_FP64, PRECISION_MIXED, PauliString, QuantumState
    from stab_decomp_simulator_rust_gb300 import workloads as W
    from stab_decomp_simulator_rust_gb300.state import counts_to_xy, xy_to_float
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
    t0 = time.perf_counter()
    counts, scale = st.exp_value_counts(zs)
    ms_exact = (time.perf_counter() - t0) * 1e3
    shots = cfg["shots"]
    ms_samp, (vals, cnts) = _timed(torch, stream, lambda: st.sample_raw(qargs, shots, seed=cfg["seed"]), 1)
    clocks.stop()

    def walsh(e):
        e = list(e)
        h = 1
        while h < 256:
            for i in range(0, 256, 2 * h):
                for j in range(i, i + h):
                    a, b = e[j], e[j + h]
                    e[j], e[j + h] = a + b, a - b
            h *= 2
        return e

    def marginal(e):
        w = walsh(np.asarray(e, float))
        return np.maximum(np.asarray(w) / (256.0 * e[0]), 0.0)
    xy = [counts_to_xy(c) for c in counts]
    wx, wy = walsh([x for x, _ in xy]), walsh([y for _, y in xy])
    X0, Y0 = xy[0]
    # p(x) = (Wx + Wy/√2) / (256·(X0 + Y0/√2)), each part rounded once from exact rationals
    den = xy_to_float(X0, Y0) * 256.0
    p_exact = np.asarray([xy_to_float(a, b) for a, b in zip(wx, wy)]) / den
    p64, pmx = marginal(e_64), marginal(e_mx)
    hist = np.zeros(256)
    for v, c in zip(vals, cnts):
        hist[v] += c
    tvd = 0.5 * float(np.abs(hist / shots - p_exact).sum())
    norm_exact = xy_to_float(X0, Y0, scale)
    line = {"metric": METRIC, "value": 256 / (ms_mx * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": 1,
            "warmup": 0, "ms_per_step": ms_mx, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 accumulation of exact pair values, f64 final reduction", "data": "synthetic (seeded generator)",
            "config": {"workload": "n=64, 8000 {H,S,CX} + 40 T (seed 5); project q0-7 onto seeded outcomes; "
                                   "1e6 samples of q8-15", "outcomes_q0_7": outcomes, "chi_compiled": chi0,
                       "chi_after_projection": chi1, "pairs_per_observable": chi1 * (chi1 + 1) // 2,
                       "compile_s": compile_s, "l2": "inputs larger than L2"},
            "stage_ms": {"project_and_renormalise": ms_proj, "norm_fp64": ms_norm,
                         "z_strings_256_mixed": ms_mx, "z_strings_256_fp64": ms_64, "z_strings_256_exact": ms_exact,
                         "sample_1e6": ms_samp},
            "norm_after_renormalise": norm, "norm_sq_exact": norm_exact, "norm_error": abs(norm - 1.0),
            "norm_sq_error_vs_exact": abs(norm * norm - norm_exact),
            "marginal_max_abs_err_vs_exact": {"mixed": float(np.abs(pmx - p_exact).max()),
                                              "fp64": float(np.abs(p64 - p_exact).max())},
            "tvd_samples_vs_exact_marginal": tvd,
            "tvd_expected_from_sampling_noise": 0.5 * float(np.sqrt(2.0 * p_exact * (1 - p_exact) / (np.pi * shots)).sum()),
            "clocks": clocks.summary()}
    print(json.dumps(line))


def run_plain40(args, torch, L):
    stream = torch.cuda.current_stream()
    r = plain40_leg(torch, stream, L, args.steps, args.warmup)
    line = {"metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
            "config": {"workload": r["workload"], "chi": r["chi"]}, "plain": r["plain"], "e2e": r["e2e"]}
    print(json.dumps(line))


def run_gates(args, torch, L):
    hbm = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))).get("hbm_gbs", 6800.0) \
        if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else 6800.0
    print(json.dumps({"workload": "gate application", "gate_apply": gate_apply_leg(torch, torch.cuda.current_stream(), hbm)}))


def run_workload(args):
    torch, L = _setup_gpu()
    {"precision60": run_precision60, "project64": run_project64, "plain40": run_plain40,
     "gates": run_gates}[args.workload](args, torch, L)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-gates", action="store_true", help="skip the gate-application leg")
    ap.add_argument("--no-plain40", action="store_true", help="skip the n=40 plain-method leg")
    ap.add_argument("--cpu-steps", type=int, default=6, help="circuits drawn for the CPU baseline in our line")
    ap.add_argument("--ref-step-seconds", type=float, default=1.5,
                    help="--impl reference: seconds of pair sampling per step")
    ap.add_argument("--plain-observables", type=int, default=4,
                    help="observables per circuit timed on the plain path (of 16)")
    ap.add_argument("--workload", default="batch512",
                    choices=["batch512", "plain40", "precision60", "project64", "gates"],
                    help="batch512: the headline line; the others one JSON line each")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch512":
        run_ours(args)
    else:
        run_workload(args)


if __name__ == "__main__":
    main()
