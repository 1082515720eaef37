"""Builds ``_build/libscf_projection.so`` (sm_103a) with nvcc.

The assembly and correction translation units are compiled with
``-fmad=false`` so that their results round exactly like the reference's
Fortran expressions; the solver units keep fused multiply-adds.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libscf_projection.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr", "-I" + CSRC]
UNITS = {
    "k_assemble.cu": ["-fmad=false"],
    "k_correct.cu": ["-fmad=false"],
    "k_solver.cu": [],
    "scf_api.cu": [],
    "k_noalloc.cu": [],
    "k_adjoint.cu": [],
    "k_cg_df.cu": [],
    "k_geometry.cu": ["-fmad=false"],
    "geo_api.cu": [],
    "k_output.cu": [],
    "k_predictor.cu": ["-fmad=false"],
    "k_bicgstab.cu": [],
    "pred_api.cu": [],
    "k_transport.cu": ["-fmad=false"],
    "scf_stage.cu": [],
}


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(unit: str, extra, verbose: bool):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(OUT, unit.replace(".cu", ".o"))
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    deps.append(os.path.join(HERE, "..", "include", "scf_projection.h"))
    deps.append(os.path.join(HERE, "..", "include", "scf_geometry.h"))
    deps.append(os.path.join(HERE, "..", "include", "scf_output.h"))
    deps.append(os.path.join(HERE, "..", "include", "scf_predictor.h"))
    deps.append(os.path.join(HERE, "..", "include", "scf_clsvof.h"))
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc(), "-c", src, "-o", obj] + ARCH + COMMON + list(extra)
    if verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stdout}\n{r.stderr}")
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], verbose), UNITS.items()))
    if os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(o) for o in objs):
        return LIB
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-Xcompiler", "-fPIC", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
