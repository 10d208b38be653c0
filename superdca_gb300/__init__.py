"""GB300 plmDCA per-locus solve engine (SuperDCA's inference step).

The compute path is the CUDA library libsuperdca_gb300.so behind the C ABI in
include/superdca_gb300.h; this package is its Python host binding plus the
alignment encoding and the seeded synthetic workloads used by the tests and
the benchmark.
"""
from ._lib import EngineError, FORM_DUAL, FORM_GATHER, FORM_TC  # noqa: F401
from .engine import Engine, SolveResult, TuneResult, autotune, coupling_lines, format_coupling_lines  # noqa: F401
