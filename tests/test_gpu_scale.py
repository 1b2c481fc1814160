"""GPU parity at the sizes the benchmark numbers come from.

* The n = 40 plain-method workload (4000 {H,S,CX} + 24 T, χ = 972): every
  term bit-exact against the oracle's compile; for 4 of its 64 observables
  the exact accumulator (signed counts of pair-term real parts per power of
  √2) equal, count for count, to the oracle's over the full χ² sum
  (stabilizer_decomposed_state/exp_value.rs:38-58), and the FP64, mixed,
  captured-plan and multi-chunk-task results within 1e-9 of the exact value.
* The n = 60 / t = 36 and n = 64 / t = 40 workloads (χ = 26,244 and 78,732,
  widths 96 and 104 during compilation): 64 sampled terms of the device
  compile bit-exact against the oracle's compile loop run on those T-tensor
  terms alone (compiler/mod.rs:92-131 is independent per term), the drop
  flags of sampled terms equal, and 64² × 3 = 12,288 pair values (k, r) of
  the sampled terms equal to the oracle's pair_scalar.
* The exact accumulator against the oracle's on small states of both row
  widths.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import random_full_circuit
from stab_decomp_simulator_rust_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-9
FIELDS = ("G", "F", "M", "gamma", "v", "s", "phase", "coef_phase", "coef_r")
BINS, MOFF = 512, 192


def close(a, b, tol=TOL):
    return abs(a - b) <= tol * max(1.0, abs(b))


def assert_same_terms(dg, dr, what=""):
    assert dg["n"] == dr["n"]
    assert len(dg["phase"]) == len(dr["phase"]), what
    for k in FIELDS:
        assert np.array_equal(dg[k], dr[k]), f"{what}: field {k} differs"


@pytest.fixture(scope="module")
def plain40(gpu_pkg, oracle):
    cfg = W.PLAIN_N40
    gates = W.random_clifford_t_circuit(cfg["n"], cfg["num_clifford"], cfg["num_t"], cfg["seed"])
    ops = W.random_dense_paulis(cfg["n"], cfg["num_paulis"], cfg["seed"] + 100)
    st = gpu_pkg.QuantumState.from_gates(cfg["n"], gates)
    ref = oracle.OracleState.from_circuit(cfg["n"], gates)
    return cfg, gates, ops, st, ref


def test_plain_n40_compile_bit_exact(plain40):
    cfg, gates, ops, st, ref = plain40
    assert st.stabilizer_rank == ref.stabilizer_rank == 972
    assert_same_terms(st.export_terms(), ref.export_terms(), "n=40 workload")


def test_plain_n40_exact_counts_and_values(gpu_pkg, oracle, plain40):
    from stab_decomp_simulator_rust_gb300.state import counts_to_value, set_pair_tiling
    cfg, gates, ops, st, ref = plain40
    pick = [0, 21, 42, 63]
    paulis = [gpu_pkg.PauliString.dense(ops[o]) for o in pick]
    want_counts, want = ref.exp_value_counts([(0, ops[o], None) for o in pick], MOFF, BINS)
    got_counts, scale = st.exp_value_counts(paulis)
    assert scale == 1.0
    assert np.array_equal(got_counts, want_counts)
    exact = [counts_to_value(c) for c in want_counts]
    for e, w in zip(exact, want):
        assert close(e, w, 1e-15)
    np.testing.assert_array_equal(st.exp_values_exact(paulis), exact)
    results = {
        "fp64": st.exp_values(paulis, gpu_pkg.PRECISION_FP64),
        "mixed": st.exp_values(paulis, gpu_pkg.PRECISION_MIXED),
        "plan": gpu_pkg.BatchPlan([st], [paulis], gpu_pkg.PRECISION_MIXED).run()[0],
        "single": [st.exp_value(p) for p in paulis],
    }
    # tilings whose tasks span several chunks (χ = 972 has ~15k chunks of 32 kets;
    # one task per resident warp makes each task cover ~7 of them)
    try:
        for chunk, tpw in ((32, 1), (8, 2), (64, 4)):
            set_pair_tiling(chunk, tpw)
            results[f"tiling{chunk}x{tpw}"] = st.exp_values(paulis, gpu_pkg.PRECISION_FP64)
    finally:
        set_pair_tiling(0, 0)
    for name, vals in results.items():
        for o, (g, e) in enumerate(zip(vals, exact)):
            assert close(g, e), (name, pick[o], g, e)


def _sampled_parity(gpu_pkg, oracle, cfg, nterms=64, seed=5):
    n = cfg["n"]
    gates = W.random_clifford_t_circuit(n, cfg["num_clifford"], cfg["num_t"], cfg["seed"])
    keep = gpu_pkg.state.compile_keep(n, gates)
    assert len(keep) == oracle.t_tensor_rank(cfg["num_t"])
    st = gpu_pkg.QuantumState.from_gates(n, gates)
    assert st.stabilizer_rank == int(keep.sum())
    rng = np.random.default_rng(seed)
    kept_idx = np.flatnonzero(keep)
    tsel = np.sort(rng.choice(kept_idx, size=min(nterms, len(kept_idx)), replace=False))
    ref, kept = oracle.OracleState.compile_terms(n, gates, tsel)
    assert kept.all(), "the oracle drops a term the device kept"
    dropped = np.flatnonzero(~keep)
    if len(dropped):
        dsel = np.sort(rng.choice(dropped, size=min(16, len(dropped)), replace=False))
        _, kd = oracle.OracleState.compile_terms(n, gates, dsel)
        assert not kd.any(), "the oracle keeps a term the device dropped"
    pos = np.searchsorted(kept_idx, tsel)  # positions of the sampled terms in the compiled state
    sub = st.select(pos)
    assert_same_terms(sub.export_terms(), ref.export_terms(), f"n={n} sampled terms")
    dense = rng.integers(0, 4, n).astype(np.uint8)
    sq = np.sort(rng.choice(n, 6, replace=False)).astype(np.uint32)
    sops = rng.integers(1, 4, 6).astype(np.uint8)
    checks = [(None, None), (gpu_pkg.PauliString.dense(dense), (0, dense, None)),
              (gpu_pkg.PauliString.sparse(sops, sq), (1, sops, sq))]
    m = len(tsel)
    npairs = 0
    for gp, op in checks:
        k, r = sub.debug_pair_values(gp)
        for i in range(m):
            for j in range(m):
                z, kk, rr = ref.pair_scalar(i, j, op)
                if z:
                    assert k[i, j] == 255, (i, j)
                else:
                    assert (k[i, j], r[i, j]) == (kk, rr), (i, j, k[i, j], r[i, j], kk, rr)
                npairs += 1
    assert npairs >= 10_000


def test_precision_n60_sampled_terms_and_pairs(gpu_pkg, oracle):
    _sampled_parity(gpu_pkg, oracle, W.PRECISION_N60)


def test_project_n64_sampled_terms_and_pairs(gpu_pkg, oracle):
    _sampled_parity(gpu_pkg, oracle, W.PROJECT_N64)


@pytest.mark.parametrize("n,nc,nt,seed", [(6, 80, 5, 31), (20, 300, 10, 32), (33, 400, 11, 33), (64, 600, 9, 34)])
def test_exact_counts_match_oracle(gpu_pkg, oracle, n, nc, nt, seed):
    gates = random_full_circuit(n, nc, nt, seed)
    st = gpu_pkg.QuantumState.from_gates(n, gates)
    ref = oracle.OracleState.from_circuit(n, gates)
    rng = np.random.default_rng(seed)
    ops = [np.zeros(n, np.uint8)] + [rng.integers(0, 4, n).astype(np.uint8) for _ in range(5)]
    ops += [rng.choice([0, 3], n).astype(np.uint8) for _ in range(3)]
    want_counts, want = ref.exp_value_counts([(0, o, None) for o in ops], MOFF, BINS)
    got_counts, _ = st.exp_value_counts([gpu_pkg.PauliString.dense(o) for o in ops])
    assert np.array_equal(got_counts, want_counts)
    got = st.exp_values_exact([gpu_pkg.PauliString.dense(o) for o in ops])
    for g, w in zip(got, want):
        assert close(g, w, 1e-15)
