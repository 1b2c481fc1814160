"""Writes kats.json: the known-answer values the reference's own tests assert.

The reference is Rust and cannot run here, so these are transcribed from its
test sources (cited per entry) or derived analytically as those tests derive
them; nothing here is computed by the code under test.

    python tests/golden/make_golden.py
"""
import json
import math
import os

HERE = os.path.dirname(os.path.abspath(__file__))


def cat_rank(m: int) -> int:
    # construct_cat_state (crates/necstar/src/state/magic_states/cat_state.rs:162-188)
    base = {1: 1, 2: 1, 3: 2, 4: 2, 5: 3, 6: 3}
    return base[m] if m in base else 3 * cat_rank(m - 4)


def main():
    r2 = 1 / math.sqrt(2)
    kats = {
        "_sources": {
            "t_tensor_rank": "2*chi_cat(t): t_state.rs:29-71 appends an X.S copy of every cat term",
            "toffoli": "stabilizer_decomposed_state/exp_value.rs:68-97, tests/test_state_calculation.py:68-82, "
                       "statevector.rs:33-49",
            "init": "tests/test_state_initialization.py:5-22",
            "doctests": "crates/necstar/src/state/mod.rs:113-129, :143-157, :297-302, :332-338, :373-384",
        },
        "t_tensor_rank": {str(t): 2 * cat_rank(t) for t in range(1, 12)},
        "toffoli": {"ZII": 0.5, "III": 1.0, "support": [0, 1, 2, 7]},
        "init": {"rank": 2, "statevector": [[r2, 0.0], [0.0, 0.0], [0.0, 0.0], [0.5, 0.5]]},
        "doctests": {"h_cx_t_amp0": 0.70710678, "h_cx_t_amp3": [0.5, 0.5], "plus_minus_ip": 0.70710678,
                     "bell_zz": 1.0, "bell_unnormalized_norm": 0.70710678},
    }
    with open(os.path.join(HERE, "kats.json"), "w") as f:
        json.dump(kats, f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main()
