"""CPU oracle for the stabilizer-decomposition path — test infrastructure only.

A C++ restatement of the reference's Rust algorithms (``necstar_oracle.cpp``),
built by ``build.py`` and bound by ``pyoracle.py``.  Only the tests,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use it.
"""
