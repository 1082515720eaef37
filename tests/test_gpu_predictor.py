"""GPU parity of the momentum predictor's implicit solves
(include/scf_predictor.h) against the oracle (oracle/predictor.c): Dp bit for
bit, Pred%u/v/w within the solve tolerance, the boundary planes and the
untouched entries exactly; FP64 and mixed precision; error paths."""
import numpy as np
import pytest

from simcoflow3d_gb300 import capi, geometry as GM, predictor as PR
from simcoflow3d_gb300.projection import ScfError
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASES = [
    ("sphere16", lambda: O.grid_preprocess(GM.geometry_inputs("c1", n=16)), {}),
    ("sphere32_lowre", lambda: O.grid_preprocess(GM.geometry_inputs("c1", n=32)), {"rey": 20.0}),
    ("cylinder_stretched", lambda: O.grid_preprocess(GM.geometry_inputs("c4", n=8)), {}),
    ("box_odd", lambda: O.grid_preprocess(GM.geometry_inputs("box", shape=(13, 9, 11), solid=None)), {}),
    ("slab", lambda: O.grid_preprocess(GM.geometry_inputs("box", shape=(19, 13, 37), solid=("xslab", 0.23))),
     {"rey": 50.0}),
]


@pytest.fixture(scope="module")
def lib(gpu_lib):
    return gpu_lib


def _run_both(inp, opts, seed=3):
    rng = np.random.default_rng(seed)
    shp = inp.shape_g()
    init = [np.asfortranarray(rng.normal(size=shp)) for _ in range(3)]
    pred_o = [a.copy(order="F") for a in init]
    dp_o = [np.asfortranarray(rng.normal(size=shp)) for _ in range(3)]
    O.predict_solves(inp, opts, pred_o, dp_o)
    pred_g = [a.copy(order="F") for a in init]
    dp_g = [np.asfortranarray(rng.normal(size=shp)) for _ in range(3)]
    ps = PR.PredictSolves(inp.imax, inp.jmax, inp.kmax)
    _, _, st = ps(inp, opts, pred_g, dp_g)
    return init, (pred_o, dp_o), (pred_g, dp_g), st


def _touched(c, I, J, K):
    m = np.zeros((I + 2, J + 2, K + 2), bool)
    if c == 0:
        m[:, 1:-1, 1:-1] = True
    elif c == 1:
        m[1:-1, :, 1:-1] = True
    else:
        m[1:-1, 1:-1, :] = True
    return m


@pytest.mark.parametrize("prec", [capi.SCF_PREC_FP64, capi.SCF_PREC_MIXED], ids=["fp64", "mixed"])
@pytest.mark.parametrize("name,make,kw", CASES, ids=[c[0] for c in CASES])
def test_predict_solves_parity(lib, name, make, kw, prec):
    inp = PR.momentum_inputs(make(), vof_old_noise=0.01, **kw)
    opts = PR.default_opts(precision=prec, rel_tol=1e-12)
    init, (po, do), (pg, dg), st = _run_both(inp, opts)
    I, J, K = inp.imax, inp.jmax, inp.kmax
    assert all(st["converged"]) and max(st["rel_residual"]) <= 1e-12
    assert st["gpu_launches"] > 10
    for c in range(3):
        # Dp: every entry bit for bit
        assert np.array_equal(dg[c].view(np.int64), do[c].view(np.int64)), c
        # Pred: untouched entries keep their values, the rest within tolerance
        t = _touched(c, I, J, K)
        assert np.array_equal(pg[c][~t], init[c][~t])
        scale = np.abs(po[c][t]).max()
        err = np.abs(pg[c][t] - po[c][t]).max()
        assert err <= 1e-9 * scale, (c, err, scale)
        # solid cells are exactly 0 in both
        ct = inp.comps[c].arrays["cell_type"]
        assert (pg[c][1:-1, 1:-1, 1:-1][ct == 2] == 0.0).all()


def test_split_api_and_device_fields(lib):
    inp = PR.momentum_inputs(O.grid_preprocess(GM.geometry_inputs("c1", n=16)))
    opts = PR.default_opts()
    ps = PR.PredictSolves(inp.imax, inp.jmax, inp.kmax)
    ps.stage(inp)
    s1 = ps.run(opts)
    s2 = ps.run(opts)   # a rerun on the same staged inputs is identical
    assert s1["iterations"] == s2["iterations"]
    pred, dp = PR.new_outputs(inp, fill=5.0)
    ps.fetch(pred, dp)
    po, do, _ = O.predict_solves(inp, opts)
    for c in range(3):
        assert np.array_equal(dp[c], do[c])
    ptrs = ps.device_fields()
    assert all(p for p in ptrs)


def test_error_paths(lib):
    inp = PR.momentum_inputs(O.grid_preprocess(GM.geometry_inputs("c1", n=8)))
    ps = PR.PredictSolves(inp.imax, inp.jmax, inp.kmax)
    with pytest.raises(ScfError) as e:
        ps.run(PR.default_opts())
    assert e.value.status == capi.SCF_ERR_NO_SOLVE
    bad = PR.momentum_inputs(O.grid_preprocess(GM.geometry_inputs("c1", n=8)))
    bad.comps[1].extcell += 3
    with pytest.raises(ScfError) as e:
        ps(bad, PR.default_opts())
    assert e.value.status == capi.SCF_ERR_BAD_INPUT
    bad = PR.momentum_inputs(O.grid_preprocess(GM.geometry_inputs("c1", n=8)))
    bad.comps[2].arrays["posnu"][0, 0, 0] = -1
    with pytest.raises(ScfError) as e:
        ps(bad, PR.default_opts())
    assert e.value.status == capi.SCF_ERR_BAD_INPUT
    o = PR.default_opts()
    o.dt = 0.0
    with pytest.raises(ScfError) as e:
        ps(inp, o)
    assert e.value.status == capi.SCF_ERR_BAD_ARG


def test_not_converged_is_reported(lib):
    inp = PR.momentum_inputs(O.grid_preprocess(GM.geometry_inputs("c1", n=16)), rey=5.0)
    o = PR.default_opts(rel_tol=1e-14, max_iter=1)
    ps = PR.PredictSolves(inp.imax, inp.jmax, inp.kmax)
    with pytest.raises(ScfError) as e:
        ps(inp, o)
    assert e.value.status == capi.SCF_ERR_NOT_CONVERGED


@pytest.mark.timeout(300)
@pytest.mark.parametrize("field", ["df_ew", "flux_div"])
@pytest.mark.parametrize("prec", [capi.SCF_PREC_FP64, capi.SCF_PREC_MIXED], ids=["fp64", "mixed"])
def test_non_finite_input_ends_the_solve(lib, field, prec):
    """A NaN in a matrix coefficient (a diffusive flux weight) or in the
    right-hand side (the flux divergence) of one cell makes the first
    BiCGStab step of a round break down.  The solve must end with an error
    status, not restart from the same residual again and again."""
    import time
    inp = PR.momentum_inputs(O.grid_preprocess(GM.geometry_inputs("c1", n=12)))
    a = inp.comps[0].arrays[field]
    a[tuple(n // 2 for n in a.shape)] = np.nan
    ps = PR.PredictSolves(inp.imax, inp.jmax, inp.kmax)
    t0 = time.perf_counter()
    with pytest.raises(ScfError) as e:
        ps(inp, PR.default_opts(precision=prec))
    assert e.value.status in (capi.SCF_ERR_NONFINITE, capi.SCF_ERR_BAD_INPUT), e.value.status
    assert time.perf_counter() - t0 < 30.0
    # the context stays usable
    ok = PR.momentum_inputs(O.grid_preprocess(GM.geometry_inputs("c1", n=12)))
    ps(ok, PR.default_opts(precision=prec))


@pytest.mark.parametrize("prec", [capi.SCF_PREC_FP64, capi.SCF_PREC_MIXED], ids=["fp64", "mixed"])
def test_dirichlet_faces_and_tiny_grid(lib, prec):
    """All six faces Dirichlet with seeded boundary values (and stronger
    cut-face terms) on the sphere, and the smallest box: Dp bit for bit,
    Pred within tolerance."""
    rng = np.random.default_rng(11)
    cases = [PR.momentum_inputs(O.grid_preprocess(GM.geometry_inputs("c1", n=12)), vof_old_noise=0.02, edf=0.5),
             PR.momentum_inputs(O.grid_preprocess(GM.geometry_inputs("box", shape=(3, 2, 4), solid=None)))]
    for c in cases[0].comps:
        c.bc_flag[:] = [0] * 6
        c.bc_var[:] = [np.asfortranarray(rng.normal(size=v.shape)) for v in c.bc_var]
    for inp in cases:
        opts = PR.default_opts(precision=prec, rel_tol=1e-12)
        init, (po, do), (pg, dg), st = _run_both(inp, opts)
        assert all(st["converged"])
        for c in range(3):
            assert np.array_equal(dg[c].view(np.int64), do[c].view(np.int64)), c
            t = _touched(c, inp.imax, inp.jmax, inp.kmax)
            assert np.array_equal(pg[c][~t], init[c][~t])
            assert np.abs(pg[c][t] - po[c][t]).max() <= 1e-9 * np.abs(po[c][t]).max()
