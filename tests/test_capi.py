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


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(scf_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib_path():
    from simcoflow3d_gb300 import build
    return build.build()


def test_library_exports_every_declared_function(lib_path):
    lib = C.CDLL(lib_path)
    names = declared_functions()
    assert len(names) >= 18
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
