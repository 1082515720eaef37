"""Generates the golden fixtures of tests/test_oracle.py.

Each fixture is the oracle's output on a small seeded workload: PoCoef and
the right-hand side (bit-exact pins of the coefficient and rhs restatement)
and the solution/corrected velocities (pinned to 1e-8).  Run from the repo
root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from simcoflow3d_gb300 import workloads as W  # noqa: E402


def build_case(case: str):
    if case == "c1_12_quirks":
        w = W.config("c1", n=12, random_tvar=True, perturb_vof_old=0.05)
        w.bcu_flag, w.bcv_flag, w.bcw_flag = (1, 0, 1, 0, 1, 0), (0, 1, 0, 1, 0, 1), (1, 1, 0, 0, 1, 1)
        w.bcu_const, w.bcv_const = (0.01, -0.02, 0.03, 0.0, 0.05, -0.01), (0.0, 0.02, -0.03, 0.04, 0.0, 0.01)
        w.bcw_const, w.bcp_const = (0.02, 0.0, 0.01, -0.02, 0.0, 0.03), (0.0,) * 6
        return w
    if case == "c4_8_dirichlet_top":
        return W.config("c4", n=8)
    raise KeyError(case)


def main():
    from oracle import oracle as O
    for case in ("c1_12_quirks", "c4_8_dirichlet_top"):
        w = build_case(case)
        ref = O.project(w, solver="csr", rel_tol=1e-13)
        np.savez_compressed(os.path.join(HERE, f"{case}.npz"), pocoef=ref["pocoef"], rhs=ref["b"], x=ref["x"],
                            u=ref["u"], v=ref["v"], w=ref["w"], p=ref["p"])
        print(case, "written")


if __name__ == "__main__":
    main()
