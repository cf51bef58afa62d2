"""The 2-D scene loader: a scene JSON in the schema of the reference's
scenes/2D/*.json (SimState<2>::load, src/simulation_state.cpp:43-60) to a
Tri2dSpec, and the loaded scene stepping on the 2-D oracle."""
import json
import os

import numpy as np
import pytest

from mfem_gb300 import abi
from mfem_gb300.meshgen import enu_to_lame, square_grid
from mfem_gb300.scene_json import SceneError, load_scene_2d, read_obj, write_dmat, write_obj


def _scene(tmp_path, **top):
    V, T = square_grid(8, 2, 0.125)
    V3 = np.concatenate([V, np.full((len(V), 1), 0.5)], axis=1)
    V3 = np.concatenate([V3, [[9.0, 9.0, 9.0]]])         # an unreferenced vertex
    write_obj(os.path.join(tmp_path, "sheet.obj"), V3, T)
    args = {
        "dt": 0.0333, "body_force": [0.0, -9.8, 0.0], "time_integrator": "BDF1",
        "linear_solver": "cholmod", "max_newton_iterations": 4,
        "objects": [{"path": "sheet.obj", "offset": [1.0, 2.0, 7.0], "material_index": 0,
                     "boundary_condition": {"type": "hangends", "ratio": 0.01, "axis": 0}}],
        "material_models": [{"youngs_modulus": 1e5, "poissons_ratio": 0.45, "density": 1e3,
                             "energy": "Stable-Neohookean"}],
        "mixed_variables": ["mixed-stretch"], "variables": []}
    args.update(top)
    p = os.path.join(tmp_path, "square.json")
    with open(p, "w") as f:
        json.dump(args, f)
    return p, V, T


def test_obj_reader_fans_polygons_and_negative_indices(tmp_path):
    p = os.path.join(tmp_path, "q.obj")
    with open(p, "w") as f:
        f.write("# quad\nv 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nf 1/1/1 2/2/2 3/3/3 4/4/4\nf -4 -3 -1\n")
    V, T = read_obj(p)
    assert V.shape == (4, 3)
    assert T.tolist() == [[0, 1, 2], [0, 2, 3], [0, 1, 3]]


def test_load_scene_2d_fields(tmp_path):
    p, V, T = _scene(tmp_path)
    sp = load_scene_2d(p)
    assert sp.V_rest.shape == V.shape and np.allclose(sp.V_rest, V + [1.0, 2.0])
    assert np.array_equal(sp.tris, T)
    lam, mu = enu_to_lame(1e5, 0.45)
    assert np.allclose(sp.mu, mu) and np.allclose(sp.lam, lam)
    assert sp.bc_type == abi.BC_HANGENDS and sp.bc_ratio == 0.01
    assert sp.body_force == (0.0, float(np.float32(-9.8)))
    # cholmod runs as the Jacobi PCG at 1e-10
    assert sp.linear_solver == abi.SOLVER_EIGEN_CG_DIAG and sp.iterative_solver_tolerance == 1e-10


def test_loaded_scene_steps_on_the_oracle(tmp_path):
    import oracle
    p, V, _ = _scene(tmp_path)
    o = oracle.OracleTri2d(load_scene_2d(p))
    for _ in range(2):
        assert o.step().status == abi.OK
    assert o.get_state()["x"][:, 1].min() < V[:, 1].min() + 2.0


def test_initial_state_and_transformation(tmp_path):
    p, V, T = _scene(tmp_path)
    x0 = V + [1.0, 2.0] + 0.01
    write_dmat(os.path.join(tmp_path, "x0.dmat"), x0)
    args = json.load(open(p))
    args["initial_state"] = {"x_path": "x0.dmat"}
    args["objects"][0]["transformation"] = [2.0, 0.0, 0.0, 1.0]
    sp = load_scene_2d(args, base_dir=str(tmp_path))
    assert np.allclose(sp.V_init, x0)
    c = (V + [1.0, 2.0]).mean(axis=0)
    assert np.allclose(sp.V_rest[:, 0] - c[0], 2 * (V[:, 0] + 1.0 - c[0]))


@pytest.mark.parametrize("change,msg", [
    (dict(material_models=[{"energy": "Neohookean"}]), "3-vector"),
    (dict(material_models=[{"energy": "Fung"}]), "3-vector"),
    (dict(variables=["stretch"]), "mixed-stretch"),
    (dict(linear_solver="minres-indefinite-block"), "not on the 2-D"),
])
def test_refusals(tmp_path, change, msg):
    p, _, _ = _scene(tmp_path, **change)
    with pytest.raises(SceneError, match=msg):
        load_scene_2d(p)


def test_clockwise_triangles_are_refused(tmp_path):
    V, T = square_grid(2, 2, 0.1)
    write_obj(os.path.join(tmp_path, "cw.obj"), V, T[:, [0, 2, 1]])
    args = {"objects": [{"path": "cw.obj"}]}
    with pytest.raises(SceneError, match="clockwise"):
        load_scene_2d(args, base_dir=str(tmp_path))
