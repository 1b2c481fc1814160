"""GPU tests of the captured batched evaluation (nsg_plan_*, BatchPlan): the
CUDA-graph replay gives the same values as the direct batched call and the
oracle, sees Clifford gates applied in place, refuses states whose rank or
width changed, and reports the tuned kernel variant."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import random_full_circuit

pytestmark = pytest.mark.gpu

TOL = 1e-9


def close_arrays(a, b, tol=TOL):
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and bool(np.all(np.abs(a - b) <= tol * np.maximum(1.0, np.abs(b))))


def make_batch(pkg, specs):
    states, plists, gates = [], [], []
    for n, nc, nt, seed, k in specs:
        g = random_full_circuit(n, nc, nt, seed)
        rng = np.random.default_rng(seed)
        states.append(pkg.QuantumState.from_gates(n, g))
        plists.append([pkg.PauliString.dense(rng.integers(0, 4, n)) for _ in range(k)])
        gates.append(g)
    return states, plists, gates


SPECS = [(5, 80, 6, 301, 7), (20, 300, 10, 302, 33), (33, 400, 8, 303, 12), (40, 500, 11, 304, 64),
         (12, 200, 9, 305, 0)]


@pytest.mark.parametrize("precision", [0, 1])
def test_plan_matches_direct_and_oracle(gpu_pkg, oracle, precision):
    states, plists, gates = make_batch(gpu_pkg, SPECS)
    plan = gpu_pkg.BatchPlan(states, plists, precision)
    direct = gpu_pkg.exp_values_multi(states, plists, precision)
    for _ in range(2):  # replays are repeatable
        got = plan.run()
        for c in range(len(states)):
            assert close_arrays(got[c], direct[c], 1e-12), c
    for c, (spec, g) in enumerate(zip(SPECS, gates)):
        if not plists[c]:
            continue
        ref = oracle.OracleState.from_circuit(spec[0], g)
        for o in (0, len(plists[c]) - 1):
            _, ex = ref.exp_value(0, plists[c][o].ops)
            assert abs(got[c][o] - ex) <= TOL * max(1.0, abs(ex)), (c, o)
    t = plan.tiling
    for w in ("rows32", "rows64"):  # SPECS has states of both row widths
        assert t[f"minb_{w}"] in ((2, 3, 4, 5, 6) if w == "rows32" else (2, 3, 4, 5))
        assert t[f"chunk_{w}"] in (16, 32, 64) and t[f"tasks_per_warp_{w}"] in (16, 64, 256)


def test_plan_sees_gates_applied_in_place(gpu_pkg):
    states, plists, _ = make_batch(gpu_pkg, SPECS[:4])
    plan = gpu_pkg.BatchPlan(states, plists)
    before = plan.run()
    rng = np.random.default_rng(7)
    for s in states:
        n = s.num_qubits
        for _ in range(20):  # Cliffords only: rank and width unchanged
            q = int(rng.integers(n))
            kind = int(rng.integers(3))
            if kind == 0:
                s.apply_h(q)
            elif kind == 1:
                s.apply_s(q)
            elif n > 1:
                s.apply_cx(q, (q + 1) % n)
    after = plan.run()
    fresh = gpu_pkg.exp_values_multi(states, plists)
    changed = False
    for c in range(len(states)):
        assert close_arrays(after[c], fresh[c], 1e-12), c
        changed |= not close_arrays(after[c], before[c], 1e-6)
    assert changed


def test_plan_refuses_changed_states(gpu_pkg):
    from stab_decomp_simulator_rust_gb300 import NecstarError
    states, plists, _ = make_batch(gpu_pkg, SPECS[:2])
    plan = gpu_pkg.BatchPlan(states, plists)
    plan.run()
    states[0].project_unnormalized(0, False)
    with pytest.raises(NecstarError) as e:
        plan.run()
    assert e.value.code == 18


def test_plan_tuning_cache(gpu_pkg):
    states, plists, _ = make_batch(gpu_pkg, [(40, 500, 11, 311, 16)])
    p1 = gpu_pkg.BatchPlan(states, plists)
    p2 = gpu_pkg.BatchPlan(states, plists)  # same device and workload class
    assert not p2.tiling["timed"]
    assert p2.tiling == dict(p1.tiling, timed=False)
    assert close_arrays(p1.run()[0], p2.run()[0], 1e-12)


_CACHE_CHILD = r"""
import json, sys
sys.path.insert(0, {root!r})
import numpy as np
import stab_decomp_simulator_rust_gb300 as pkg
from stab_decomp_simulator_rust_gb300 import workloads as W
g = W.random_clifford_t_circuit(36, 500, 12, 313)
st = pkg.QuantumState.from_gates(36, g)
ps = [pkg.PauliString.dense(p) for p in W.random_dense_paulis(36, 24, 314)]
plan = pkg.BatchPlan([st], [ps])
print(json.dumps(plan.tiling))
"""


def test_plan_tuning_cache_file_round_trip(gpu_pkg, tmp_path):
    """NSG_TUNE_CACHE: a first process times the candidates and appends its
    choice (variant, tasks per warp, chunk); a second process reads it back
    and takes the same tiling without timing."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    cache = tmp_path / "tune.jsonl"
    env = dict(os.environ, NSG_TUNE_CACHE=str(cache))
    code = _CACHE_CHILD.format(root=root)
    first = json.loads(subprocess.run([sys.executable, "-c", code], env=env, check=True, capture_output=True,
                                      text=True).stdout.strip().splitlines()[-1])
    lines = [json.loads(x) for x in cache.read_text().splitlines()]
    assert first["timed"] and len(lines) == 1
    assert {"key", "minb", "tasks_per_warp", "chunk"} <= set(lines[0])
    assert (lines[0]["minb"], lines[0]["tasks_per_warp"], lines[0]["chunk"]) == \
        (first["minb_rows64"], first["tasks_per_warp_rows64"], first["chunk_rows64"])
    second = json.loads(subprocess.run([sys.executable, "-c", code], env=env, check=True, capture_output=True,
                                       text=True).stdout.strip().splitlines()[-1])
    assert not second["timed"]
    assert second == dict(first, timed=False)


def test_empty_plan(gpu_pkg):
    plan = gpu_pkg.BatchPlan([], [])
    assert plan.run() == []
