"""GB300-native pressure projection for SIMCOFlow (Simcoflow3D).

The package wraps ``libscf_projection.so`` (hand-written sm_103a CUDA behind a
C ABI that mirrors ``PoissonEquationSolver``/``UpdatePUVW``) and provides the
synthetic workloads used by the tests and the benchmark.
"""
