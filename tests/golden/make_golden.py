"""Generates the committed golden fixtures in this directory.

kat_dRdF.json
    The inputs of the reference's "dRdF" test (tests/test_dsvd.cpp:204-238):
    F = 2*Matrix3d::Random(), S = Matrix3d::Random() as Eigen 3.4 draws them
    in a fresh process (std::rand() with the default seed 1, mapped to
    -1 + 2*rand()/RAND_MAX, column-major fill).  The glibc rand() stream is
    reproduced by calling libc here.  The test passes when
    |dRdF_fd - dRdF| <= 1e-5 with central differences of step 1e-5.
kat_dsvd.json
    The fixed F of tests/test_dsvd.cpp:74-110.
c1_oracle_fp64.npz
    Positions of the FP64 oracle on the 200-tet beam after 1, 10 and 100
    steps (a regression pin of the oracle itself).
tri2d_oracle_fp64.npz
    Positions of the FP64 2-D oracle on a 10 x 3 hanging sheet (60
    triangles, the settings of scenes/2D/square.json) after 1 and 10 steps
    (a regression pin of the 2-D oracle).

Run from the repository root:  python tests/golden/make_golden.py
"""
import ctypes
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)


def eigen_random3(libc):
    RAND_MAX = 2147483647
    m = np.zeros((3, 3))
    for c in range(3):
        for r in range(3):
            m[r, c] = -1.0 + 2.0 * libc.rand() / RAND_MAX
    return m


def tri2d_sheet_spec():
    from mfem_gb300 import abi
    from mfem_gb300.desc import Tri2dSpec
    from mfem_gb300.meshgen import enu_to_lame, square_grid
    V, T = square_grid(10, 3, 0.1)
    lam, mu = enu_to_lame(1e5, 0.45)
    return Tri2dSpec(V_rest=V, tris=T, mu=np.full(len(T), mu), lam=np.full(len(T), lam),
                     density_const=1000.0, bc_type=abi.BC_HANGENDS, bc_ratio=0.01, bc_axis=0,
                     dt=0.0333, max_newton_iterations=4, iterative_solver_tolerance=1e-12,
                     max_iterative_solver_iters=10000)


def write_tri2d():
    import oracle
    sc = oracle.OracleTri2d(tri2d_sheet_spec())
    out = {}
    for step in range(1, 11):
        sc.step()
        if step in (1, 10):
            out[f"x_{step}"] = sc.get_state()["x"]
    np.savez_compressed(os.path.join(HERE, "tri2d_oracle_fp64.npz"), **out)


def main():
    libc = ctypes.CDLL("libc.so.6")
    libc.srand(1)
    F = 2.0 * eigen_random3(libc)
    S = eigen_random3(libc)
    with open(os.path.join(HERE, "kat_dRdF.json"), "w") as f:
        json.dump({"source": "tests/test_dsvd.cpp:204-238", "F": F.tolist(), "S": S.tolist(),
                   "alpha": 1e-5, "tol": 1e-8, "max_iter": 200, "bound": 1e-5}, f, indent=1)
    Fd = [[1.0, 0.1, 0.2], [0.1, 2.0, 0.4], [0.3, 0.4, 0.5]]
    with open(os.path.join(HERE, "kat_dsvd.json"), "w") as f:
        json.dump({"source": "tests/test_dsvd.cpp:74-110", "F": Fd}, f, indent=1)

    import oracle
    from mfem_gb300 import configs
    sc = oracle.OracleScene(configs.beam_c1())
    out = {}
    for step in range(1, 101):
        sc.step()
        if step in (1, 10, 100):
            out[f"x_{step}"] = sc.get_state()["x"]
    np.savez_compressed(os.path.join(HERE, "c1_oracle_fp64.npz"), **out)
    write_tri2d()
    print("written")


if __name__ == "__main__":
    main()
