"""The device V-cycle against the oracle's CPU V-cycle (oracle/gmg.cpp):
same hierarchy rule, Chebyshev smoother (point-Jacobi or 8-cell z-line
blocks) and coarse solve, applied to a seeded residual.  FP64 V-cycle to
1e-12, FP32 V-cycle to 2e-5 (relative L2), on cubes, an odd-sized box and the
Dirichlet-top wave tank; the 64^3 case takes the large-level path (separate
prolongation and first post-smoothing step)."""
import numpy as np
import pytest

from simcoflow3d_gb300 import workloads as W

pytestmark = pytest.mark.gpu

CASES = [("c1", dict(n=24)), ("c2", dict(n=24)), ("c4", dict(n=12)), ("odd", {}), ("c1", dict(n=64))]


def _workload(name, kw):
    if name == "odd":
        return W.build_workload("odd", 37, 13, 21, solid=W.SPHERE_C1, liquid=("bubble", 0.5, 0.5, 0.6, 0.2),
                                rho_l=1000.0, rho_g=1.2)
    return W.config(name, **kw)


@pytest.mark.parametrize("lines", [0, 1])
@pytest.mark.parametrize("degree", [2, 3, 4])
@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 2e-5)])
@pytest.mark.parametrize("name,kw", CASES)
def test_vcycle_matches_oracle(gpu_lib, name, kw, precision, tol, degree, lines):
    from oracle import oracle as O
    from simcoflow3d_gb300.projection import Projection
    w = _workload(name, kw)
    p = Projection.for_workload(w, rel_tol=1e-6, precision=precision, smoother_degree=degree,
                                smoother_lines=lines)
    pc, _, _ = p.poisson_solve(w)
    act = np.zeros(w.shape_g, dtype=bool)
    act[1:-1, 1:-1, 1:-1] = w.arrays["cell_type"] != 2
    rng = np.random.default_rng(17)
    for trial in range(2):
        r = np.where(act, rng.normal(size=w.shape_g), 0.0)
        if all(f == 1 for f in w.bcp_flag):
            r[act] -= r[act].mean()
        r = np.asfortranarray(r)
        z = p.debug_precondition(r)
        zr = O.gmg_vcycle(w, pc, r, precision=0, degree=degree, line_seg=8 if lines else 0)
        err = np.linalg.norm(z - zr) / np.linalg.norm(zr)
        assert err <= tol, (trial, err)
        assert not z[~act].any()
