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


def _big_odd(n0=70, n1=45, n2=85):
    # 70 x 45 x 85 = 267,750 cells: a large level whose tiles are ragged in
    # every direction (70 = 2*32 + 6, 45 = 5*8 + 5, 85 = 2*32 + 21)
    return W.build_workload("odd-large", n0, n1, n2, solid=W.SPHERE_C1, liquid=("bubble", 0.5, 0.5, 0.6, 0.2),
                            rho_l=1000.0, rho_g=1.2)


# Row lengths n0 + 2 of both residues mod 4 that the two-step kernel's
# row-pair view takes: 72 (odd rows start on a 16-byte boundary, n1 may be
# odd) and 70 (odd rows start 8 bytes past one, n1 even); 68 x 46 x 85 =
# 266,016 cells, tiles ragged in every direction too.
@pytest.mark.parametrize("shape", [(70, 45, 85), (68, 46, 85)])
@pytest.mark.parametrize("degree", [2, 3, 4, 5])
def test_paired_smoother_equals_one_step_sweeps(gpu_lib, degree, shape):
    """The two-step kernel (one pass per pair of Chebyshev steps), forced
    onto every level of at least 2^18 cells, gives the V-cycle and the
    projection of one-step sweeps bit for bit, whatever the k-planes per
    block."""
    from simcoflow3d_gb300.projection import Projection, smoother_pair_counts, smoother_pairs
    w = _big_odd(*shape)
    act = np.zeros(w.shape_g, dtype=bool)
    act[1:-1, 1:-1, 1:-1] = w.arrays["cell_type"] != 2
    r = np.where(act, np.random.default_rng(5).normal(size=w.shape_g), 0.0)
    r[act] -= r[act].mean()
    r = np.asfortranarray(r)
    out = {}
    try:
        for key, on, planes in (("one", 0, 0), ("pairs", 2, 0), ("pairs7", 2, 7), ("pairs1", 2, 1)):
            smoother_pairs(on, planes)
            p = Projection.for_workload(w, rel_tol=1e-8, precision=1, smoother_degree=degree, smoother_lines=0)
            _, pp, st = p.poisson_solve(w, want_pocoef=False)
            out[key] = (p.debug_precondition(r), pp, st["iterations"])
            p.close()
    finally:
        smoother_pairs(1, 0)
    # the fused runs went through the TMA-staged kernel, with no fallback
    tma, fallback = smoother_pair_counts()
    assert tma > 0 and fallback == 0, (tma, fallback)
    z0, p0, n0 = out["one"]
    for key in ("pairs", "pairs7", "pairs1"):
        z, pp, n = out[key]
        assert np.array_equal(z, z0), key
        assert n == n0 and np.array_equal(pp, p0), key
