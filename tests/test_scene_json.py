"""Scene JSON loader (the reference's schema, src/simulation_state.cpp:92-366)."""
import json

import numpy as np
import pytest

from mfem_gb300 import abi
from mfem_gb300.meshgen import cube_grid, enu_to_lame
from mfem_gb300.scene_json import (SceneError, load_scene, read_dmat, read_mesh, write_dmat,
                                   write_mesh)


def _files(tmp_path):
    V, T = cube_grid(4, 1, 1, 0.1)
    write_mesh(tmp_path / "beam.mesh", V, T)
    ids = (np.arange(len(T)) % 2).astype(float)
    write_dmat(tmp_path / "ids.dmat", ids)
    return V, T, ids


def _scene(**kw):
    d = {
        "dt": 0.01, "body_force": [0.0, -9.8, 0.0], "max_newton_iterations": 7,
        "max_linesearch_iterations": 12, "max_iterative_solver_iters": 300,
        "iterative_solver_tolerance": 1e-7, "time_integrator": "BDF2",
        "linear_solver": "eigen-pcg-diag", "optimizer": "newton",
        "mixed_variables": ["mixed-stretch"],
        "material_models": [
            {"youngs_modulus": 1e6, "poissons_ratio": 0.45, "density": 1000, "energy": "Stable-Neohookean"},
            {"youngs_modulus": 2e5, "poissons_ratio": 0.3, "density": 1000, "energy": "Corot"}],
        "objects": [{"path": "beam.mesh", "material_ids": "ids.dmat",
                     "boundary_condition": {"type": "hang", "axis": 0}}],
    }
    d.update(kw)
    return d


def test_mesh_and_dmat_round_trip(tmp_path):
    V, T, ids = _files(tmp_path)
    V2, T2 = read_mesh(tmp_path / "beam.mesh")
    assert np.array_equal(V, V2) and np.array_equal(T, T2)
    assert np.array_equal(read_dmat(tmp_path / "ids.dmat").ravel(), ids)
    M = np.arange(12.0).reshape(4, 3)
    write_dmat(tmp_path / "m.dmat", M)
    assert np.array_equal(read_dmat(tmp_path / "m.dmat"), M)


def test_load_scene_fields(tmp_path):
    V, T, ids = _files(tmp_path)
    p = tmp_path / "scene.json"
    p.write_text(json.dumps(_scene()))
    s = load_scene(str(p))
    assert s.n_vertices == len(V) and s.n_tets == len(T)
    lam0, mu0 = enu_to_lame(1e6, 0.45)
    lam1, mu1 = enu_to_lame(2e5, 0.3)
    assert np.allclose(s.mu, np.where(ids == 0, mu0, mu1))
    assert np.allclose(s.lam, np.where(ids == 0, lam0, lam1))
    assert list(s.material) == [abi.MATERIAL_SNH if i == 0 else abi.MATERIAL_COROT for i in ids]
    assert s.bc_type == abi.BC_HANG and s.bdf_order == 2 and s.dt == 0.01
    assert s.max_newton_iterations == 7 and s.max_linesearch_iterations == 12
    assert s.linear_solver == abi.SOLVER_EIGEN_CG_DIAG and s.iterative_solver_tolerance == 1e-7
    assert s.body_force[1] == float(np.float32(-9.8))  # SimConfig::ext is float


def test_offset_transformation_velocity_and_defaults(tmp_path):
    V, T, _ = _files(tmp_path)
    A = [2.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0]
    d = {"objects": [{"path": "beam.mesh", "offset": [1.0, 2.0, 3.0], "transformation": A,
                      "initial_velocity": [0.5, 0.0, 0.0]}]}
    s = load_scene(d, base_dir=str(tmp_path))
    Vo = V + [1.0, 2.0, 3.0]
    c = Vo.mean(axis=0)
    assert np.allclose(s.V_rest, (Vo - c) @ np.diag([2.0, 1.0, 1.0]).T + c)
    assert np.allclose(s.v_init, [0.5, 0.0, 0.0])
    # reference defaults: eigen-llt -> the GPU PCG at 1e-10, SNH E=1e6 nu=0.45, BDF1
    assert s.linear_solver == abi.SOLVER_EIGEN_CG_DIAG and s.iterative_solver_tolerance == 1e-10
    assert s.bdf_order == 1 and s.dt == 0.034 and s.max_newton_iterations == 5
    with pytest.raises(SceneError):
        load_scene(d, base_dir=str(tmp_path), direct_solver="error")


def test_two_objects_are_concatenated(tmp_path):
    V, T, _ = _files(tmp_path)
    d = {"objects": [{"path": "beam.mesh"}, {"path": "beam.mesh", "offset": [0, 1, 0]}],
         "linear_solver": "gpu-pcg-block"}
    s = load_scene(d, base_dir=str(tmp_path))
    assert s.n_vertices == 2 * len(V) and s.n_tets == 2 * len(T)
    assert s.tets[len(T):].min() == len(V)
    assert s.linear_solver == abi.SOLVER_GPU_PCG_BLOCK


def test_rejections(tmp_path):
    _files(tmp_path)
    with pytest.raises(SceneError):
        load_scene(_scene(mixed_variables=["stretch"]), base_dir=str(tmp_path))
    with pytest.raises(SceneError):
        load_scene(_scene(variables=["stretch"]), base_dir=str(tmp_path))  # both variables
    fem = _scene(variables=["stretch"])
    del fem["mixed_variables"]
    assert load_scene(fem, base_dir=str(tmp_path)).formulation == abi.FORMULATION_STRETCH
    with pytest.raises(SceneError):
        load_scene(_scene(linear_solver="minres-indefinite-admm"), base_dir=str(tmp_path))
    s = load_scene(_scene(linear_solver="minres-indefinite-block"), base_dir=str(tmp_path))
    assert s.linear_solver == abi.SOLVER_MINRES_ID
    two = _scene()
    two["objects"] = [{"path": "beam.mesh", "boundary_condition": {"type": "hang"}},
                      {"path": "beam.mesh", "boundary_condition": {"type": "twist"}}]
    with pytest.raises(SceneError):
        load_scene(two, base_dir=str(tmp_path))
    bad = _scene()
    bad["objects"][0] = {"path": "beam.mesh", "material_index": 5}
    with pytest.raises(SceneError):
        load_scene(bad, base_dir=str(tmp_path))


def test_loaded_scene_steps_like_the_built_one_in_the_oracle(tmp_path):
    import oracle
    from mfem_gb300.desc import SceneSpec
    V, T, ids = _files(tmp_path)
    s = load_scene(_scene(), base_dir=str(tmp_path), precision=abi.PRECISION_FP64)
    lam0, mu0 = enu_to_lame(1e6, 0.45)
    lam1, mu1 = enu_to_lame(2e5, 0.3)
    direct = SceneSpec(V_rest=V, tets=T, mu=np.where(ids == 0, mu0, mu1),
                       lam=np.where(ids == 0, lam0, lam1),
                       material=np.where(ids == 0, abi.MATERIAL_SNH, abi.MATERIAL_COROT).astype(np.int32),
                       bc_type=abi.BC_HANG, bc_axis=0, dt=0.01,
                       body_force=(0.0, float(np.float32(-9.8)), 0.0), bdf_order=2,
                       max_newton_iterations=7, max_linesearch_iterations=12,
                       max_iterative_solver_iters=300, iterative_solver_tolerance=1e-7,
                       precision=abi.PRECISION_FP64)
    a, b = oracle.OracleScene(s), oracle.OracleScene(direct)
    for _ in range(3):
        a.step()
        b.step()
    assert np.array_equal(a.get_state()["x"], b.get_state()["x"])
