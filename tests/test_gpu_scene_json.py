"""A scene loaded from the reference's JSON schema steps on the GPU as in the oracle."""
import json

import numpy as np
import pytest

from mfem_gb300 import abi
from mfem_gb300.meshgen import cube_grid
from mfem_gb300.scene_json import load_scene, write_dmat, write_mesh


@pytest.mark.gpu
def test_json_scene_gpu_matches_oracle(gpu_lib, tmp_path):
    import oracle
    from mfem_gb300 import gpu
    V, T = cube_grid(6, 2, 2, 0.1)
    write_mesh(tmp_path / "beam.mesh", V, T)
    write_dmat(tmp_path / "ids.dmat", (np.arange(len(T)) % 2).astype(float))
    scene = {
        "dt": 0.01, "max_newton_iterations": 10, "iterative_solver_tolerance": 1e-10,
        "max_iterative_solver_iters": 2000, "linear_solver": "eigen-pcg-diag",
        "material_models": [{"youngs_modulus": 1e5, "poissons_ratio": 0.4, "energy": "Stable-Neohookean"},
                            {"youngs_modulus": 3e5, "poissons_ratio": 0.3, "energy": "Neohookean"}],
        "objects": [{"path": "beam.mesh", "material_ids": "ids.dmat",
                     "boundary_condition": {"type": "hang", "axis": 0}}],
    }
    (tmp_path / "scene.json").write_text(json.dumps(scene))
    spec = load_scene(str(tmp_path / "scene.json"), precision=abi.PRECISION_FP64)
    g, o = gpu.Scene(spec), oracle.OracleScene(spec)
    for _ in range(10):
        g.step()
        o.step()
    xg, xo = g.get_state()["x"], o.get_state()["x"]
    diag = np.linalg.norm(xo.max(axis=0) - xo.min(axis=0))
    assert np.abs(xg - xo).max() <= 1e-6 * diag
