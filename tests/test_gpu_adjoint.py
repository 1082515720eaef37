"""GPU adjoint of the projection loss: against the FP64 reference gradient
of the oracle (oracle/adjoint.py), against central finite differences on 32
seeded random directions (eps = 1e-6) at 128^3 on the c1 geometry, and
through torch.autograd."""
import numpy as np
import pytest

from simcoflow3d_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _runner(w, **kw):
    from simcoflow3d_gb300.autograd import ProjectionLoss
    return ProjectionLoss(w, **kw)


def test_adjoint_matches_fp64_reference_gradient(gpu_lib):
    from oracle import adjoint as AD
    w = W.config("c1", n=14)
    g = W.pressure_force_weights(w)
    rng = np.random.default_rng(4)
    rho = AD.phase_density(w) * np.exp(0.1 * rng.normal(size=w.shape_g))
    rho = np.asfortranarray(rho)
    Jr, gr, grho_r = AD.gradient(w, rho, g)
    R = _runner(w, g=g)
    J, parts, _ = R.forward(w.arrays["u_star"], w.arrays["v_star"], w.arrays["w_star"], rho)
    (gu, gv, gw, grho), _ = R.backward()
    assert abs(J - Jr) <= 1e-9 * abs(Jr)
    for a, b in zip((gu, gv, gw), gr):
        assert np.linalg.norm(a - b) <= 1e-8 * np.linalg.norm(b)
    assert np.linalg.norm(grho - grho_r) <= 1e-8 * np.linalg.norm(grho_r)


def test_adjoint_phase_densities_reproduce_reference_forward(gpu_lib):
    """With rho = NULL the loss uses the reference's own coefficients."""
    from simcoflow3d_gb300.projection import Projection
    w = W.config("c1", n=16)
    g = W.pressure_force_weights(w)
    R = _runner(w, g=g)
    J, (Jp, Jd), _ = R.forward(w.arrays["u_star"], w.arrays["v_star"], w.arrays["w_star"], None)
    p = Projection.for_workload(w, rel_tol=1e-12)
    _, pp, _ = p.poisson_solve(w)
    assert abs(Jp - float(np.sum(g * pp[1:-1, 1:-1, 1:-1]))) <= 1e-10 * abs(Jp)


def test_adjoint_finite_differences_128(gpu_lib):
    """32 seeded directions for (u*, v*, w*) and 32 for rho, central
    differences with eps = 1e-6.  The error is relative to the size of the
    directional derivatives over the set of directions: a single random
    direction can be nearly orthogonal to the gradient, where a per-direction
    relative error says nothing."""
    from oracle import adjoint as AD
    w = W.config("c3", n=128)
    g = W.pressure_force_weights(w)
    rho = AD.phase_density(w)
    R = _runner(w, g=g)
    a = w.arrays
    us, vs, ws = a["u_star"], a["v_star"], a["w_star"]
    R.forward(us, vs, ws, rho)
    (gu, gv, gw, grho), _ = R.backward()
    rng = np.random.default_rng(20261203)
    eps = 1.0e-6
    fd_u, an_u, fd_r, an_r = [], [], [], []
    for _ in range(32):
        d = [np.asfortranarray(rng.normal(size=w.shape_g)) for _ in range(3)]
        Jp = R.forward(us + eps * d[0], vs + eps * d[1], ws + eps * d[2], rho)[0]
        Jm = R.forward(us - eps * d[0], vs - eps * d[1], ws - eps * d[2], rho)[0]
        fd_u.append((Jp - Jm) / (2 * eps))
        an_u.append(float(np.sum(gu * d[0]) + np.sum(gv * d[1]) + np.sum(gw * d[2])))
    for _ in range(32):
        dr = np.asfortranarray(rng.normal(size=w.shape_g) * rho)
        Jp = R.forward(us, vs, ws, rho + eps * dr)[0]
        Jm = R.forward(us, vs, ws, rho - eps * dr)[0]
        fd_r.append((Jp - Jm) / (2 * eps))
        an_r.append(float(np.sum(grho * dr)))
    for fd, an in ((fd_u, an_u), (fd_r, an_r)):
        fd, an = np.array(fd), np.array(an)
        assert np.linalg.norm(fd - an) <= 1e-6 * np.linalg.norm(an), (fd, an)
        assert np.abs(fd - an).max() <= 2e-6 * np.abs(an).max(), (fd, an)
    # The density directions' residual error at eps = 1e-6 is rounding of the
    # FP64 operator amplified by its conditioning and divided by 2 eps (it
    # scales as 1/eps); at eps = 1e-5 it is ten times smaller.
    eps = 1.0e-5
    rng = np.random.default_rng(20261204)
    fd_r, an_r = [], []
    for _ in range(8):
        dr = np.asfortranarray(rng.normal(size=w.shape_g) * rho)
        Jp = R.forward(us, vs, ws, rho + eps * dr)[0]
        Jm = R.forward(us, vs, ws, rho - eps * dr)[0]
        fd_r.append((Jp - Jm) / (2 * eps))
        an_r.append(float(np.sum(grho * dr)))
    fd, an = np.array(fd_r), np.array(an_r)
    assert np.linalg.norm(fd - an) <= 3e-7 * np.linalg.norm(an), (fd, an)


def test_torch_autograd_function(gpu_lib):
    import torch
    from simcoflow3d_gb300.autograd import ProjectionLoss, projection_loss, _to_t
    from oracle import adjoint as AD
    w = W.config("c1", n=12)
    R = ProjectionLoss(w)
    a = w.arrays
    u = _to_t(a["u_star"]).clone().requires_grad_(True)
    v = _to_t(a["v_star"]).clone().requires_grad_(True)
    ww = _to_t(a["w_star"]).clone().requires_grad_(True)
    rho = _to_t(AD.phase_density(w)).clone().requires_grad_(True)
    J = projection_loss(u, v, ww, rho, R)
    (2.0 * J).backward()
    (gu, gv, gw, grho), _ = R.backward()
    assert torch.allclose(u.grad, 2.0 * _to_t(gu), rtol=0, atol=0)
    assert torch.allclose(rho.grad, 2.0 * _to_t(grho), rtol=0, atol=0)
