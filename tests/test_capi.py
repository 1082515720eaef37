"""The C ABI library builds for sm_103a, loads, exports every function the
header declares, and the ctypes mirror matches the C struct layouts.  No
device calls (runs without a GPU)."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "scf_projection.h")
GEO_HEADER = os.path.join(ROOT, "include", "scf_geometry.h")
OUT_HEADER = os.path.join(ROOT, "include", "scf_output.h")
PRED_HEADER = os.path.join(ROOT, "include", "scf_predictor.h")
CLSVOF_HEADER = os.path.join(ROOT, "include", "scf_clsvof.h")


def declared_functions():
    names = set()
    for h in (HEADER, GEO_HEADER, OUT_HEADER, PRED_HEADER, CLSVOF_HEADER):
        src = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        names |= set(re.findall(r"\b(scf_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


@pytest.fixture(scope="module")
def lib_path():
    from simcoflow3d_gb300 import build
    return build.build()


def test_library_exports_every_declared_function(lib_path):
    lib = C.CDLL(lib_path)
    names = declared_functions()
    assert len(names) >= 25
    assert "scf_grid_preprocess" in names and "scf_geo_create" in names and "scf_write_vtr" in names
    assert "scf_predict_solves" in names and "scf_mom_run" in names
    assert "scf_clsvof_step" in names and "scf_clsvof_run" in names
    for n in names:
        assert hasattr(lib, n), n
    assert lib.scf_abi_version() == 2


def test_struct_layouts_match_header(lib_path):
    from simcoflow3d_gb300 import capi
    prog = r'''
#include <stdio.h>
#include <stddef.h>
#include "scf_projection.h"
#define P(T, f) printf(#T " " #f " %zu\n", offsetof(T, f));
int main(void) {
  printf("scf_opts size %zu\n", sizeof(scf_opts));
  printf("scf_stats size %zu\n", sizeof(scf_stats));
  printf("scf_poisson_in size %zu\n", sizeof(scf_poisson_in));
  printf("scf_correct_in size %zu\n", sizeof(scf_correct_in));
  printf("scf_bc_out size %zu\n", sizeof(scf_bc_out));
  P(scf_opts, time_limit_s) P(scf_opts, stale_init) P(scf_stats, bytes_d2h) P(scf_stats, ms_total)
  P(scf_poisson_in, bcp_flag) P(scf_poisson_in, bcp_var) P(scf_poisson_in, dt)
  P(scf_correct_in, bcp_const) P(scf_correct_in, bcu_flag)
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "l.c")
        open(c, "w").write(prog)
        exe = os.path.join(d, "l")
        subprocess.run(["gcc", "-I", os.path.dirname(HEADER), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    got = {}
    for line in out.splitlines():
        t, f, v = line.split()
        got[(t, f)] = int(v)
    m = {"scf_opts": capi.ScfOpts, "scf_stats": capi.ScfStats, "scf_poisson_in": capi.ScfPoissonIn,
         "scf_correct_in": capi.ScfCorrectIn, "scf_bc_out": capi.ScfBcOut}
    for (t, f), v in got.items():
        if f == "size":
            assert C.sizeof(m[t]) == v, (t, v)
        else:
            assert getattr(m[t], f).offset == v, (t, f, v)


def test_product_does_not_reach_the_oracle():
    """Nothing in the shipped package imports, links or loads the oracle."""
    pkg = os.path.join(ROOT, "simcoflow3d_gb300")
    for dp, _, files in os.walk(pkg):
        for fn in files:
            if fn.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
                txt = open(os.path.join(dp, fn)).read()
                for pat in ("import oracle", "from oracle", "liboracle", "oracle/"):
                    assert pat not in txt, (fn, pat)


def test_geometry_struct_layouts_match_header():
    from simcoflow3d_gb300 import capi
    prog = r'''
#include <stdio.h>
#include <stddef.h>
#include "scf_geometry.h"
#define P(T, f) printf(#T " " #f " %zu\n", offsetof(T, f));
int main(void) {
  printf("scf_geo_cells size %zu\n", sizeof(scf_geo_cells));
  printf("scf_geo_stats size %zu\n", sizeof(scf_geo_stats));
  P(scf_geo_cells, vof) P(scf_geo_cells, cell_type) P(scf_geo_cells, fce) P(scf_geo_cells, moexcell)
  P(scf_geo_cells, posnu) P(scf_geo_cells, ext_cell)
  P(scf_geo_stats, exact_faces) P(scf_geo_stats, ms_h2d) P(scf_geo_stats, bytes_d2h) P(scf_geo_stats, ms_faces)
  P(scf_geo_stats, bytes_faces)
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "g.c")
        open(c, "w").write(prog)
        exe = os.path.join(d, "g")
        subprocess.run(["gcc", "-I", os.path.dirname(GEO_HEADER), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    m = {"scf_geo_cells": capi.ScfGeoCells, "scf_geo_stats": capi.ScfGeoStats}
    lines = out.splitlines()
    assert len(lines) == 13
    for line in lines:
        t, f, v = line.split()
        if f == "size":
            assert C.sizeof(m[t]) == int(v), (t, v)
        else:
            assert getattr(m[t], f).offset == int(v), (t, f, v)


def test_predictor_struct_layouts_match_header():
    from simcoflow3d_gb300 import capi
    prog = r'''
#include <stdio.h>
#include <stddef.h>
#include "scf_predictor.h"
#define P(T, f) printf(#T " " #f " %zu\n", offsetof(T, f));
int main(void) {
  printf("scf_mom_in size %zu\n", sizeof(scf_mom_in));
  printf("scf_mom_opts size %zu\n", sizeof(scf_mom_opts));
  printf("scf_mom_stats size %zu\n", sizeof(scf_mom_stats));
  P(scf_mom_in, cell_type) P(scf_mom_in, extcell) P(scf_mom_in, vof_old) P(scf_mom_in, tvar)
  P(scf_mom_in, bc_flag) P(scf_mom_in, bc_var)
  P(scf_mom_opts, beta_vis) P(scf_mom_opts, max_iter) P(scf_mom_opts, precision)
  P(scf_mom_stats, rel_residual) P(scf_mom_stats, ms_assemble) P(scf_mom_stats, bytes_d2h)
  P(scf_mom_stats, gpu_launches) P(scf_mom_stats, ms_kernels) P(scf_mom_opts, kernel_timing)
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "m.c")
        open(c, "w").write(prog)
        exe = os.path.join(d, "m")
        subprocess.run(["gcc", "-I", os.path.dirname(PRED_HEADER), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    m = {"scf_mom_in": capi.ScfMomIn, "scf_mom_opts": capi.ScfMomOpts, "scf_mom_stats": capi.ScfMomStats}
    lines = out.splitlines()
    assert len(lines) == 18
    for line in lines:
        t, f, v = line.split()
        if f == "size":
            assert C.sizeof(m[t]) == int(v), (t, v)
        else:
            assert getattr(m[t], f).offset == int(v), (t, f, v)


def test_clsvof_struct_layouts_match_header():
    from simcoflow3d_gb300 import capi
    prog = r'''
#include <stdio.h>
#include <stddef.h>
#include "scf_clsvof.h"
#define P(T, f) printf(#T " " #f " %zu\n", offsetof(T, f));
int main(void) {
  printf("scf_clsvof_in size %zu\n", sizeof(scf_clsvof_in));
  printf("scf_clsvof_state size %zu\n", sizeof(scf_clsvof_state));
  printf("scf_clsvof_stats size %zu\n", sizeof(scf_clsvof_stats));
  P(scf_clsvof_in, u) P(scf_clsvof_in, bc_w_b) P(scf_clsvof_in, lvs_flag) P(scf_clsvof_in, vof_flag)
  P(scf_clsvof_in, lvs_const) P(scf_clsvof_in, vof_const) P(scf_clsvof_in, dt)
  P(scf_clsvof_state, nzl) P(scf_clsvof_state, lvs_bc) P(scf_clsvof_state, vof_bc)
  P(scf_clsvof_stats, bytes_h2d) P(scf_clsvof_stats, steps) P(scf_clsvof_stats, gpu_launches)
  P(scf_clsvof_stats, ms_kernels)
  printf("scf_clsvof_vcell size %zu\n", sizeof(scf_clsvof_vcell));
  P(scf_clsvof_vcell, phil) P(scf_clsvof_vcell, vofl)
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "m.c")
        open(c, "w").write(prog)
        exe = os.path.join(d, "m")
        subprocess.run(["gcc", "-I", os.path.dirname(CLSVOF_HEADER), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    m = {"scf_clsvof_in": capi.ScfClsvofIn, "scf_clsvof_state": capi.ScfClsvofState,
         "scf_clsvof_stats": capi.ScfClsvofStats, "scf_clsvof_vcell": capi.ScfClsvofVcell}
    lines = out.splitlines()
    assert len(lines) == 20
    for line in lines:
        t, f, v = line.split()
        if f == "size":
            assert C.sizeof(m[t]) == int(v), (t, v)
        else:
            assert getattr(m[t], f).offset == int(v), (t, f, v)


def test_noalloc_size_guard_rejects_huge_grids_before_any_launch(lib_path):
    """The allocation-free apply checks the ghosted size in 64-bit arithmetic:
    I + 2 near INT32_MAX must not wrap to a small or negative count.  The guard
    returns SCF_ERR_BAD_ARG before any CUDA call, so this runs without a GPU."""
    from simcoflow3d_gb300 import capi
    lib = C.CDLL(lib_path)
    f = lib.scf_apply_operator_noalloc
    f.argtypes = [C.c_int32, C.c_int32, C.c_int32] + [C.c_void_p] * 8
    f.restype = C.c_int
    dummy = C.c_void_p(16)   # never dereferenced: the size guard comes first
    big = 2 ** 31 - 1
    for dims in ((big, 1, 1), (1, big, 1), (1, 1, big), (big, big, big), (2 ** 20, 2 ** 20, 2 ** 20)):
        rc = f(*dims, dummy, dummy, dummy, dummy, dummy, dummy, None, None)
        assert rc == capi.SCF_ERR_BAD_ARG, dims
    assert f(0, 4, 4, dummy, dummy, dummy, dummy, dummy, dummy, None, None) == capi.SCF_ERR_BAD_ARG
