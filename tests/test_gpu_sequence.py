"""A sequence of projections on a fixed geometry (the wave-tank workload:
512x256x256 in full, here 2n x n x n, z-stretched, vertical cylinder, free
surface, Dirichlet-p top): each call gets a freshly seeded prediction and
starts from the previous call's pressure.  Every call must reach the
tolerance in both precisions, the warm-started pressure must match a cold
FP64 solve of the same call, warm starts must not cost iterations, and the
first and last calls' pressure and corrected velocity must match the
oracle's projection of the same prediction (FP64 solve to 1e-13,
ComputePUVW.f90:179-384)."""
import numpy as np
import pytest

from simcoflow3d_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _oracle_call(w, pred):
    """The oracle's projection of workload ``w`` with (u*, v*, w*) = pred."""
    wp = w.copy()
    for key, a in zip(("u_star", "v_star", "w_star"), pred):
        wp.arrays[key] = np.asfortranarray(a)
    return O.project(wp, rel_tol=1e-13)


@pytest.mark.parametrize("precision", [0, 1])
def test_warm_started_sequence_wave_tank(gpu_lib, precision):
    from simcoflow3d_gb300.projection import Projection
    w = W.config("c4", n=24)
    assert w.bcp_flag[5] == 0
    seq = Projection.for_workload(w, rel_tol=1e-8, precision=precision, warm_start=1)
    cold = Projection.for_workload(w, rel_tol=1e-8, precision=0)
    act = w.arrays["cell_type"] != 2
    its_warm, its_cold = [], []
    for call in range(20):
        pred = W.perturbed_prediction(w, seed=4000 + call)
        seq.stage(w, pred=pred)
        st = seq.run()
        assert st["converged"] == 1 and st["rel_residual"] <= 1e-8
        its_warm.append(st["iterations"])
        pw = np.zeros(w.shape_g, order="F")
        uvw = [np.zeros(w.shape_g, order="F") for _ in range(3)]
        seq.fetch(*uvw, pp=pw)
        if call in (0, 19):
            ref = _oracle_call(w, pred)
            assert ref["stats"]["csr_relres"] <= 2e-13
            err_p = O.pressure_error(w, pw, ref["pp"], ref["singular"])
            err_u = O.velocity_error(uvw, (ref["u"], ref["v"], ref["w"]))
            assert err_p <= 1e-5 and err_u <= 1e-6, (call, err_p, err_u)
        cold.stage(w, pred=pred)
        sc = cold.run()
        its_cold.append(sc["iterations"])
        pc = np.zeros(w.shape_g, order="F")
        cold.fetch(pp=pc)
        d = (pw - pc)[1:-1, 1:-1, 1:-1][act]
        assert np.abs(d).max() <= 1e-5 * np.abs(pc[1:-1, 1:-1, 1:-1][act]).max(), call
    assert sum(its_warm[1:]) <= sum(its_cold[1:])


@pytest.mark.parametrize("stretched", [True, False])
def test_smoother_blocks_follow_the_grid(gpu_lib, stretched):
    """smoother_lines=2 (default) takes 8-cell z-line blocks on a strongly
    z-stretched grid and single cells on a uniform one, in mixed precision:
    its pressure is bitwise that of the explicit choice.  Line blocks also
    cut the iterations on the stretched grid."""
    from simcoflow3d_gb300.projection import Projection
    if stretched:
        w = W.build_workload("stretched", 32, 32, 32, zstretch=1.4, solid=W.SPHERE_C1,
                             liquid=("bubble", 0.5, 0.5, 0.6, 0.2), rho_l=1000.0, rho_g=1.2)
    else:
        w = W.config("c1", n=32)
    out = {}
    for lines in (2, 1, 0):
        p = Projection.for_workload(w, rel_tol=1e-8, precision=1, smoother_lines=lines)
        _, pp, st = p.poisson_solve(w, want_pocoef=False)
        assert st["converged"] == 1
        out[lines] = (pp, st["iterations"])
    expect = 1 if stretched else 0
    assert np.array_equal(out[2][0], out[expect][0])
    if stretched:
        assert out[1][1] < out[0][1]
