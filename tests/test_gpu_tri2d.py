"""The 2-D path on the GPU (mfem_gpu_tri2d_*) against the 2-D oracle:
the element update (polar_svd<2>, materials, Aloc), the assembled system,
whole timesteps under every BC script and material, BDF2, and
run-to-run bitwise reproducibility."""
import ctypes as C

import numpy as np
import pytest

from mfem_gb300 import abi
from mfem_gb300.desc import Tri2dSpec, make_tri2d_desc
from mfem_gb300.meshgen import enu_to_lame, square_grid


def spec2(nx=10, ny=3, spacing=0.1, E=1e5, nu=0.45, seed=None, **kw):
    V, T = square_grid(nx, ny, spacing)
    lam, mu = enu_to_lame(E, nu)
    args = dict(V_rest=V, tris=T, mu=np.full(len(T), mu), lam=np.full(len(T), lam),
                density_const=1000.0, bc_type=abi.BC_HANGENDS, bc_ratio=0.01, bc_axis=0,
                dt=0.0333, max_newton_iterations=3, iterative_solver_tolerance=1e-10)
    if seed is not None:
        rng = np.random.default_rng(seed)
        args["V_init"] = V + 0.2 * spacing * rng.uniform(-1, 1, V.shape)
    args.update(kw)
    return Tri2dSpec(**args)


def test_tri2d_desc_layout_matches_header():
    from tests.test_abi import _c_layout
    fields = [n for n, _ in abi.Tri2dDesc._fields_]
    got = _c_layout("mfem_tri2d_desc", ["lambda" if f == "lam" else f for f in fields])
    assert got[0] == C.sizeof(abi.Tri2dDesc)
    for f, off in zip(fields, got[1:]):
        assert getattr(abi.Tri2dDesc, f).offset == off, f


def test_no_device_fails_loudly_without_gpu(gpu_lib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    d = make_tri2d_desc(spec2(3, 2))
    h = C.c_void_p()
    assert gpu_lib.mfem_gpu_tri2d_create(C.addressof(d.struct), C.byref(h)) == abi.ERR_NO_DEVICE


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.gpu
@pytest.mark.parametrize("mtype", [abi.MATERIAL_SNH, abi.MATERIAL_COROT, abi.MATERIAL_FCR,
                                   abi.MATERIAL_ARAP])
def test_elem_update_matches_oracle(gpu_lib, mtype):
    import oracle
    from mfem_gb300.tri2d import Tri2dScene
    # a perturbed initial state, so that s (= polar(F(V_init))) is away
    # from the rest value and g = h^2 grad psi(s) is not rounding noise
    sp = spec2(6, 3, seed=11, material=np.full(36, mtype, np.int32))
    o, g = oracle.OracleTri2d(sp), Tri2dScene(sp)
    rng = np.random.default_rng(7)
    x = sp.V_rest * np.array([1.1, 0.95]) + 0.03 * rng.uniform(-1, 1, sp.V_rest.shape)
    ro, rg = o.elem_update(x, 0.02), g.elem_update(x, 0.02)
    for k in ("R", "S", "dSdF", "g", "H", "Aloc", "gl"):
        assert _rel(rg[k], ro[k]) < 1e-10, k
    # Where the psd projection clamps two eigenvalues of an SNH Hessian to
    # 1e-6 next to one near 1e6 (condition 1e12), the cofactor 3x3 inverse
    # (Eigen's Matrix3d::inverse, which both sides restate) returns rounding
    # noise on either side; H^-1 is compared where H's condition is below
    # 1e8, with that condition times rounding as the tolerance.
    Ho = ro["H"].reshape(-1, 3, 3)
    ok = np.linalg.cond(Ho) < 1e8
    assert ok.sum() >= len(ok) // 2
    assert _rel(rg["Hinv"][ok], ro["Hinv"][ok]) < 1e-7
    g.close()


@pytest.mark.gpu
def test_system_matches_oracle(gpu_lib):
    import oracle
    from mfem_gb300.tri2d import Tri2dScene
    sp = spec2(8, 3, seed=3)
    o, g = oracle.OracleTri2d(sp), Tri2dScene(sp)
    rpo, co, vo, bo = o.get_system()
    rpg, cg, vg, bg = g.get_system()
    assert np.array_equal(rpo, rpg) and np.array_equal(co, cg)
    assert _rel(vg, vo) < 1e-11
    assert _rel(bg, bo) < 1e-10
    g.close()


def _bbox(x):
    return float(np.linalg.norm(x.max(axis=0) - x.min(axis=0)))


def _run_pair(sp, steps):
    import oracle
    from mfem_gb300.tri2d import Tri2dScene
    o, g = oracle.OracleTri2d(sp), Tri2dScene(sp)
    for _ in range(steps):
        so, sg = o.step(), g.step()
        assert sg.status == so.status
        assert sg.newton_iterations == so.newton_iterations
    return o.get_state(), g.get_state(), g


@pytest.mark.gpu
@pytest.mark.parametrize("mtype", [abi.MATERIAL_SNH, abi.MATERIAL_COROT, abi.MATERIAL_FCR,
                                   abi.MATERIAL_ARAP])
def test_steps_match_oracle(gpu_lib, mtype):
    sp = spec2(12, 3, material=np.full(72, mtype, np.int32))
    so, sg, g = _run_pair(sp, 6)
    scale = _bbox(so["x"])
    assert np.abs(sg["x"] - so["x"]).max() < 1e-8 * scale
    assert np.abs(sg["v"] - so["v"]).max() < 1e-6 * max(np.abs(so["v"]).max(), 1e-3)
    assert np.abs(sg["s"] - so["s"]).max() < 1e-7
    assert np.abs(so["x"] - sp.V_rest).max() > 1e-3 * scale   # it moved
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("bc", [abi.BC_STRETCH, abi.BC_TWIST, abi.BC_BEND, abi.BC_HANG,
                                abi.BC_COMPRESS])
def test_bc_scripts_match_oracle(gpu_lib, bc):
    """(SCALEF is left out: the 1.5x blown-up sheet's line search fails by
    halving to rounding-level energy differences, which no two summation
    orders need to resolve alike.)"""
    sp = spec2(8, 2, bc_type=bc, bc_ratio=0.1, bc_velocity=0.2)
    so, sg, g = _run_pair(sp, 3)
    assert np.abs(sg["x"] - so["x"]).max() < 1e-8 * _bbox(so["x"])
    g.close()


@pytest.mark.gpu
def test_bdf2_matches_oracle(gpu_lib):
    sp = spec2(10, 3, bdf_order=2)
    so, sg, g = _run_pair(sp, 5)
    assert np.abs(sg["x"] - so["x"]).max() < 1e-8 * _bbox(so["x"])
    g.close()


@pytest.mark.gpu
def test_runs_are_bitwise_reproducible(gpu_lib):
    from mfem_gb300.tri2d import Tri2dScene
    sp = spec2(16, 4, seed=5)
    out = []
    for _ in range(2):
        g = Tri2dScene(sp)
        for _ in range(3):
            g.step()
        out.append(g.get_state())
        g.close()
    for k in ("x", "v", "s", "R"):
        assert np.array_equal(out[0][k], out[1][k]), k


@pytest.mark.gpu
def test_scene_json_2d_runs_on_gpu_like_the_oracle(gpu_lib, tmp_path):
    """A scene file in the 2-D schema through the loader, on both sides."""
    import json
    import os
    import oracle
    from mfem_gb300.scene_json import load_scene_2d, write_obj
    from mfem_gb300.tri2d import Tri2dScene
    V, T = square_grid(8, 2, 0.125)
    write_obj(os.path.join(tmp_path, "sheet.obj"), V, T)
    scene = {"dt": 0.0333, "linear_solver": "cholmod", "max_newton_iterations": 3,
             "objects": [{"path": "sheet.obj",
                          "boundary_condition": {"type": "hangends", "ratio": 0.01}}],
             "material_models": [{"youngs_modulus": 1e5, "poissons_ratio": 0.45,
                                  "energy": "Stable-Neohookean"}]}
    p = os.path.join(tmp_path, "s.json")
    json.dump(scene, open(p, "w"))
    sp = load_scene_2d(p)
    o, g = oracle.OracleTri2d(sp), Tri2dScene(sp)
    for _ in range(3):
        assert g.step().status == o.step().status
    xo, xg = o.get_state()["x"], g.get_state()["x"]
    assert np.abs(xg - xo).max() < 1e-8 * _bbox(xo)
    g.close()


@pytest.mark.gpu
def test_large_sheet_grid_pcg_matches_oracle_and_is_reproducible(gpu_lib):
    """A sheet with more free rows (about 1070) than the one-block PCG takes
    (1024): the PCG runs over co-resident blocks (t2_pcg_grid, two grid
    barriers an iteration) and still follows the oracle within 1e-8 of the
    bounding-box diagonal, with equal Newton counts, and reruns bitwise."""
    from mfem_gb300.tri2d import Tri2dScene
    sp = spec2(64, 16, spacing=1.0 / 64, max_iterative_solver_iters=5000)
    so, sg, g = _run_pair(sp, 3)
    assert g.n_free > 1024
    assert np.abs(sg["x"] - so["x"]).max() < 1e-8 * _bbox(so["x"])
    assert np.abs(so["x"] - sp.V_rest).max() > 1e-4 * _bbox(so["x"])   # it moved
    g.close()
    out = []
    for _ in range(2):
        h = Tri2dScene(sp)
        for _ in range(2):
            h.step()
        out.append(h.get_state()["x"])
        h.close()
    assert np.array_equal(out[0], out[1])
