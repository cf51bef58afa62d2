"""Scene JSON loader: the reference's scene schema to a SceneSpec.

Follows SimState<3>::load and load_params (src/simulation_state.cpp:92-366)
with the names of the reference's factories (src/factories/*.cpp), so that a
scene file written for the reference runs on the GPU path unchanged:

  top level   dt, body_force, max_newton_iterations, max_linesearch_iterations,
              max_iterative_solver_iters, iterative_solver_tolerance,
              time_integrator ("BDF1".."BDF6"), linear_solver, optimizer,
              mixed_variables, variables, material_models, objects,
              initial_state {x_path, v_path}
  material    youngs_modulus, poissons_ratio, density, energy
              ("Stable-Neohookean", "Neohookean", "Corot", "FixedCorot",
              "ARAP", "Fung")
  object      path (.mesh), offset, transformation (3x3, column-major as
              Eigen::Map reads it), initial_velocity, material_index or
              material_ids (.dmat), boundary_condition {type, axis, ratio,
              velocity}

As in the reference's Factory (src/factories/factory.h:35-42) an unknown name
maps to the enum's first value.  Several objects are concatenated into one
scene (Meshes, src/mesh/meshes.cpp:11-56); they must share one boundary
condition script, the descriptor's single BC.

The GPU path runs the mixed-stretch variable only.  Direct solvers
("eigen-llt", "eigen-ldlt", "eigen-lu", "cholmod") have no GPU form: with
direct_solver="pcg" (the default) they become the GPU Jacobi PCG at a
relative tolerance of 1e-10, which agrees with a direct solve to that
tolerance; with direct_solver="error" the loader refuses them.
"""
import json
import os

import numpy as np

from . import abi
from .desc import SceneSpec, Tri2dSpec
from .meshgen import enu_to_lame

MATERIALS = {"Stable-Neohookean": abi.MATERIAL_SNH, "Neohookean": abi.MATERIAL_NH,
             "Corot": abi.MATERIAL_COROT, "FixedCorot": abi.MATERIAL_FCR,
             "ARAP": abi.MATERIAL_ARAP, "Fung": abi.MATERIAL_FUNG}
BCS = {"null": abi.BC_NULL, "scale": abi.BC_SCALEF, "randomize": abi.BC_RANDOM,
       "onepoint": abi.BC_ONEPOINT, "hang": abi.BC_HANG, "hangends": abi.BC_HANGENDS,
       "bend": abi.BC_BEND, "stretch": abi.BC_STRETCH, "twist": abi.BC_TWIST,
       "pinmin": abi.BC_PINMIN, "compress": abi.BC_COMPRESS}
INTEGRATORS = {f"BDF{k}": k for k in range(1, 7)}
SOLVERS = {"eigen-llt": abi.SOLVER_EIGEN_LLT, "eigen-ldlt": abi.SOLVER_EIGEN_LDLT,
           "eigen-lu": abi.SOLVER_EIGEN_LU, "cholmod": abi.SOLVER_CHOLMOD,
           "eigen-pcg-diag": abi.SOLVER_EIGEN_CG_DIAG, "eigen-pcg-IC": abi.SOLVER_EIGEN_CG_IC,
           "admm-solver": abi.SOLVER_ADMM, "minres-indefinite-block": abi.SOLVER_MINRES_ID,
           "minres-indefinite-admm": abi.SOLVER_MINRES_ADMM,
           "gpu-pcg-block": abi.SOLVER_GPU_PCG_BLOCK}
DIRECT = {abi.SOLVER_EIGEN_LLT, abi.SOLVER_EIGEN_LDLT, abi.SOLVER_EIGEN_LU, abi.SOLVER_CHOLMOD}


class SceneError(ValueError):
    """A scene file the GPU path cannot run."""


def _by_name(table, name, default):
    return table.get(name, default)


# ----------------------------------------------------------------- files --
def read_mesh(path):
    """MEDIT .mesh (what igl::readMESH reads): 'Vertices' then x y z ref,
    'Tetrahedra' then four 1-based indices and a ref.  Returns V (n,3), T (m,4)."""
    with open(path) as f:
        toks = f.read().split()
    V, T = None, None
    i = 0
    while i < len(toks):
        t = toks[i]
        if t == "Vertices":
            n = int(toks[i + 1])
            vals = np.array(toks[i + 2:i + 2 + 4 * n], dtype=np.float64).reshape(n, 4)
            V = vals[:, :3].copy()
            i += 2 + 4 * n
        elif t == "Tetrahedra":
            m = int(toks[i + 1])
            vals = np.array(toks[i + 2:i + 2 + 5 * m], dtype=np.int64).reshape(m, 5)
            T = (vals[:, :4] - 1).astype(np.int32)
            i += 2 + 5 * m
        elif t in ("Triangles", "Edges", "Corners", "Ridges", "RequiredVertices"):
            n = int(toks[i + 1])
            width = {"Triangles": 4, "Edges": 3, "Corners": 1, "Ridges": 1, "RequiredVertices": 1}[t]
            i += 2 + width * n
        else:
            i += 1
    if V is None or T is None:
        raise SceneError(f"{path}: no vertices or tetrahedra")
    if T.min() < 0 or T.max() >= len(V):
        raise SceneError(f"{path}: tetrahedron index out of range")
    return V, T


def write_mesh(path, V, T):
    with open(path, "w") as f:
        f.write("MeshVersionFormatted 1\nDimension 3\n")
        f.write(f"Vertices\n{len(V)}\n")
        for v in V:
            f.write(f"{v[0]:.17g} {v[1]:.17g} {v[2]:.17g} 0\n")
        f.write(f"Tetrahedra\n{len(T)}\n")
        for t in T:
            f.write(f"{t[0] + 1} {t[1] + 1} {t[2] + 1} {t[3] + 1} 0\n")
        f.write("End\n")


def read_dmat(path):
    """libigl's text .dmat: 'cols rows' then the entries in column-major order."""
    with open(path) as f:
        toks = f.read().split()
    cols, rows = int(toks[0]), int(toks[1])
    vals = np.array(toks[2:2 + rows * cols], dtype=np.float64)
    return vals.reshape(cols, rows).T


def write_dmat(path, M):
    M = np.atleast_2d(np.asarray(M, dtype=np.float64))
    if M.shape[0] == 1 and M.ndim == 2 and M.size > 1:
        M = M.T
    rows, cols = M.shape
    with open(path, "w") as f:
        f.write(f"{cols} {rows}\n")
        for v in M.T.ravel():
            f.write(f"{v:.17g}\n")


# ---------------------------------------------------------------- loader --
def load_scene(src, base_dir=None, direct_solver="pcg", precision=abi.PRECISION_MIXED, **overrides):
    """Scene JSON (a path, a JSON string or a dict) to a SceneSpec.
    Relative paths in the file resolve against base_dir (default: the
    file's directory, else the current directory)."""
    if isinstance(src, dict):
        args = src
    elif isinstance(src, str) and src.lstrip().startswith("{"):
        args = json.loads(src)
    else:
        with open(src) as f:
            args = json.load(f)
        if base_dir is None:
            base_dir = os.path.dirname(os.path.abspath(src))
    base_dir = base_dir or os.getcwd()

    def path_of(p):
        return p if os.path.isabs(p) else os.path.join(base_dir, p)

    # "mixed_variables": ["mixed-stretch"] (MixedStretch) or "variables":
    # ["stretch"] (standard FEM, Stretch); a scene naming neither gets the
    # mixed-stretch variable (the reference would simulate no elasticity)
    mixed = args.get("mixed_variables")
    plain = args.get("variables") or []
    if plain:
        if list(plain) != ["stretch"] or mixed:
            raise SceneError(f"variables {plain} with mixed_variables {mixed} are not on the GPU path")
        formulation = abi.FORMULATION_STRETCH
    else:
        mixed = ["mixed-stretch"] if mixed is None else mixed
        if "mixed-stretch" not in mixed:
            raise SceneError("the GPU path runs the mixed-stretch or the stretch variable; the scene "
                             f"names {mixed}")
        formulation = abi.FORMULATION_MIXED_STRETCH

    # materials (MaterialConfig defaults, src/config.h:127-135)
    mats = []
    for m in args.get("material_models", [{}]):
        E = float(m.get("youngs_modulus", 1e6))
        nu = float(m.get("poissons_ratio", 0.45))
        lam, mu = enu_to_lame(E, nu)
        mats.append(dict(mu=float(mu), lam=float(lam), rho=float(m.get("density", 1000.0)),
                         mat=_by_name(MATERIALS, m.get("energy"), abi.MATERIAL_SNH)))

    Vs, Ts, mu, lam, rho, mat, vel, bcs = [], [], [], [], [], [], [], []
    nv = 0
    for obj in args.get("objects", []):
        if "path" not in obj:
            raise SceneError("object missing path")
        V, T = read_mesh(path_of(obj["path"]))
        V = V + np.asarray(obj.get("offset", [0.0, 0.0, 0.0]), dtype=np.float64)
        if obj.get("transformation"):
            A = np.asarray(obj["transformation"], dtype=np.float64).reshape(3, 3, order="F")
            c = V.mean(axis=0)
            V = (V - c) @ A.T + c
        if "material_ids" in obj:
            ids = read_dmat(path_of(obj["material_ids"])).ravel().astype(np.int64)
            if len(ids) != len(T) or ids.min() < 0 or ids.max() >= len(mats):
                raise SceneError("material_ids do not match the mesh or the materials")
        else:
            idx = int(obj.get("material_index", 0))
            if idx >= len(mats):
                raise SceneError("material_index out of range")
            ids = np.full(len(T), idx)
        mu.append(np.array([mats[i]["mu"] for i in ids]))
        lam.append(np.array([mats[i]["lam"] for i in ids]))
        rho.append(np.array([mats[i]["rho"] for i in ids]))
        mat.append(np.array([mats[i]["mat"] for i in ids], dtype=np.int32))
        v0 = np.zeros_like(V)
        if obj.get("initial_velocity"):
            v0[:] = np.asarray(obj["initial_velocity"], dtype=np.float64)
        vel.append(v0)
        bc = obj.get("boundary_condition")
        bcs.append(None if bc is None else (
            _by_name(BCS, bc.get("type"), abi.BC_NULL), int(bc.get("axis", 0)),
            float(bc.get("ratio", 0.1)), float(bc.get("velocity", 0.1))))
        Vs.append(V)
        Ts.append(T + nv)
        nv += len(V)
    if not Vs:
        raise SceneError("scene has no objects")
    given = [b for b in bcs if b is not None]
    if given and any(b != given[0] for b in given):
        raise SceneError("objects with different boundary conditions in one scene")
    bc = given[0] if given else (abi.BC_NULL, 0, 0.1, 0.1)

    V = np.concatenate(Vs)
    v_init = np.concatenate(vel)
    V_init = None
    init = args.get("initial_state", {})
    if "x_path" in init:
        V_init = read_dmat(path_of(init["x_path"]))
        if V_init.shape != V.shape:
            raise SceneError("initial_state x_path does not match the meshes")
    if "v_path" in init:
        v_init = read_dmat(path_of(init["v_path"]))
        if v_init.shape != V.shape:
            raise SceneError("initial_state v_path does not match the meshes")

    solver = _by_name(SOLVERS, args.get("linear_solver"), abi.SOLVER_EIGEN_LLT)
    tol = float(args.get("iterative_solver_tolerance", 1e-4))
    iters = int(args.get("max_iterative_solver_iters", 500))
    if solver in DIRECT:
        if direct_solver != "pcg":
            raise SceneError(f"direct solver {args.get('linear_solver')} has no GPU form")
        solver, tol, iters = abi.SOLVER_EIGEN_CG_DIAG, 1e-10, max(iters, 10000)
    elif solver not in (abi.SOLVER_EIGEN_CG_DIAG, abi.SOLVER_GPU_PCG_BLOCK, abi.SOLVER_MINRES_ID):
        raise SceneError(f"linear solver {args.get('linear_solver')} is not on the GPU path")

    rho_all = np.concatenate(rho)
    spec = SceneSpec(
        V_rest=V, tets=np.concatenate(Ts).astype(np.int32), mu=np.concatenate(mu),
        lam=np.concatenate(lam), V_init=V_init,
        v_init=v_init if np.any(v_init) else None, material=np.concatenate(mat),
        density=None if np.all(rho_all == rho_all[0]) else rho_all,
        density_const=float(rho_all[0]), bc_type=bc[0], bc_axis=bc[1], bc_ratio=bc[2],
        bc_velocity=bc[3], dt=float(args.get("dt", 0.034)),
        body_force=tuple(float(np.float32(v)) for v in args.get("body_force", [0.0, -9.8, 0.0])),
        bdf_order=_by_name(INTEGRATORS, args.get("time_integrator"), 1),
        max_newton_iterations=int(args.get("max_newton_iterations", 5)),
        max_linesearch_iterations=int(args.get("max_linesearch_iterations", 20)),
        max_iterative_solver_iters=iters, iterative_solver_tolerance=tol,
        linear_solver=solver, precision=precision, formulation=formulation,
        name=os.path.basename(src) if isinstance(src, str) and not src.lstrip().startswith("{") else "scene")
    for k, v in overrides.items():
        setattr(spec, k, v)
    return spec


# ------------------------------------------------------------ 2-D scenes --
def read_obj(path):
    """Wavefront .obj as igl::read_triangle_mesh reads it: 'v x y [z]' and
    'f a b c ...' (1-based, 'a/t/n' forms allowed, negative indices count
    from the end); polygons are split into fans.  Returns V (n,3), T (m,3)."""
    V, T = [], []
    with open(path) as f:
        for line in f:
            tok = line.split()
            if not tok:
                continue
            if tok[0] == "v":
                xyz = [float(t) for t in tok[1:4]]
                V.append(xyz + [0.0] * (3 - len(xyz)))
            elif tok[0] == "f":
                idx = []
                for t in tok[1:]:
                    i = int(t.split("/")[0])
                    idx.append(i - 1 if i > 0 else len(V) + i)
                for k in range(1, len(idx) - 1):
                    T.append([idx[0], idx[k], idx[k + 1]])
    if not V or not T:
        raise SceneError(f"{path}: no vertices or faces")
    V = np.asarray(V, dtype=np.float64)
    T = np.asarray(T, dtype=np.int64)
    if T.min() < 0 or T.max() >= len(V):
        raise SceneError(f"{path}: face index out of range")
    return V, T.astype(np.int32)


def write_obj(path, V, T):
    with open(path, "w") as f:
        for v in V:
            z = v[2] if len(v) > 2 else 0.0
            f.write(f"v {v[0]:.17g} {v[1]:.17g} {z:.17g}\n")
        for t in T:
            f.write(f"f {t[0] + 1} {t[1] + 1} {t[2] + 1}\n")


def load_scene_2d(src, base_dir=None, direct_solver="pcg", **overrides):
    """A 2-D scene JSON (the schema above, as SimState<2>::load reads it,
    src/simulation_state.cpp:43-60 and 92-366) to a Tri2dSpec.

    Differences from 3-D, all the reference's: meshes are triangle meshes
    read by igl::read_triangle_mesh (.obj here), unreferenced vertices are
    removed and z is dropped (no normalisation); offsets, initial velocities
    and body_force use their first two components; transformation is 2x2;
    material_ids are ignored (the reference prints "Missing heterogeneous
    2Dtrimesh support!" and uses the object's material_index).  The 2-D path
    runs the mixed-stretch variable with SNH, Corot, FixedCorot or ARAP (the
    materials with a 3-vector energy) and the Jacobi PCG; direct solvers
    become that PCG at 1e-10 as in 3-D.  Clockwise triangles (a negative
    igl::doublearea, which the reference would use as a negative weight)
    are refused."""
    if isinstance(src, dict):
        args = src
    elif isinstance(src, str) and src.lstrip().startswith("{"):
        args = json.loads(src)
    else:
        with open(src) as f:
            args = json.load(f)
        if base_dir is None:
            base_dir = os.path.dirname(os.path.abspath(src))
    base_dir = base_dir or os.getcwd()

    def path_of(p):
        return p if os.path.isabs(p) else os.path.join(base_dir, p)

    mixed = args.get("mixed_variables")
    mixed = ["mixed-stretch"] if mixed is None else mixed
    if args.get("variables") or "mixed-stretch" not in mixed:
        raise SceneError("the 2-D path runs the mixed-stretch variable only")
    mats = []
    for m in args.get("material_models", [{}]):
        E = float(m.get("youngs_modulus", 1e6))
        nu = float(m.get("poissons_ratio", 0.45))
        lam, mu = enu_to_lame(E, nu)
        mt = _by_name(MATERIALS, m.get("energy"), abi.MATERIAL_SNH)
        if mt in (abi.MATERIAL_NH, abi.MATERIAL_FUNG):
            raise SceneError(f"material {m.get('energy')} has no 3-vector (2-D) energy")
        mats.append(dict(mu=float(mu), lam=float(lam), rho=float(m.get("density", 1000.0)), mat=mt))

    Vs, Ts, mu, lam, rho, mat, vel, bcs = [], [], [], [], [], [], [], []
    nv = 0
    for obj in args.get("objects", []):
        if "path" not in obj:
            raise SceneError("object missing path")
        V3, T = read_obj(path_of(obj["path"]))
        used = np.unique(T)                      # igl::remove_unreferenced
        remap = np.full(len(V3), -1, dtype=np.int64)
        remap[used] = np.arange(len(used))
        V = V3[used, :2].copy()
        T = remap[T].astype(np.int32)
        V = V + np.asarray(obj.get("offset", [0.0, 0.0, 0.0])[:2], dtype=np.float64)
        if obj.get("transformation"):
            A = np.asarray(obj["transformation"], dtype=np.float64).reshape(2, 2, order="F")
            c = V.mean(axis=0)
            V = (V - c) @ A.T + c
        X = V[T]
        area2 = (X[:, 1, 0] - X[:, 0, 0]) * (X[:, 2, 1] - X[:, 0, 1]) - \
            (X[:, 2, 0] - X[:, 0, 0]) * (X[:, 1, 1] - X[:, 0, 1])
        if (area2 <= 0).any():
            raise SceneError(f"{obj['path']}: {int((area2 <= 0).sum())} clockwise or degenerate "
                             "triangles")
        idx = int(obj.get("material_index", 0))
        if idx >= len(mats):
            raise SceneError("material_index out of range")
        m = mats[idx]
        mu.append(np.full(len(T), m["mu"]))
        lam.append(np.full(len(T), m["lam"]))
        rho.append(np.full(len(T), m["rho"]))
        mat.append(np.full(len(T), m["mat"], dtype=np.int32))
        v0 = np.zeros_like(V)
        if obj.get("initial_velocity"):
            v0[:] = np.asarray(obj["initial_velocity"][:2], dtype=np.float64)
        vel.append(v0)
        bc = obj.get("boundary_condition")
        bcs.append(None if bc is None else (
            _by_name(BCS, bc.get("type"), abi.BC_NULL), int(bc.get("axis", 0)),
            float(bc.get("ratio", 0.1)), float(bc.get("velocity", 0.1))))
        Vs.append(V)
        Ts.append(T + nv)
        nv += len(V)
    if not Vs:
        raise SceneError("scene has no objects")
    given = [b for b in bcs if b is not None]
    if given and any(b != given[0] for b in given):
        raise SceneError("objects with different boundary conditions in one scene")
    bc = given[0] if given else (abi.BC_NULL, 0, 0.1, 0.1)
    if bc[1] not in (0, 1):
        raise SceneError("a 2-D boundary condition axis is 0 or 1")

    V = np.concatenate(Vs)
    v_init = np.concatenate(vel)
    V_init = None
    init = args.get("initial_state", {})
    if "x_path" in init:
        V_init = read_dmat(path_of(init["x_path"]))
        if V_init.shape != V.shape:
            raise SceneError("initial_state x_path does not match the meshes")
    if "v_path" in init:
        v_init = read_dmat(path_of(init["v_path"]))
        if v_init.shape != V.shape:
            raise SceneError("initial_state v_path does not match the meshes")

    solver = _by_name(SOLVERS, args.get("linear_solver"), abi.SOLVER_EIGEN_LLT)
    tol = float(args.get("iterative_solver_tolerance", 1e-4))
    iters = int(args.get("max_iterative_solver_iters", 500))
    if solver in DIRECT:
        if direct_solver != "pcg":
            raise SceneError(f"direct solver {args.get('linear_solver')} has no GPU form")
        solver, tol, iters = abi.SOLVER_EIGEN_CG_DIAG, 1e-10, max(iters, 10000)
    elif solver != abi.SOLVER_EIGEN_CG_DIAG:
        raise SceneError(f"linear solver {args.get('linear_solver')} is not on the 2-D GPU path")

    rho_all = np.concatenate(rho)
    bf = args.get("body_force", [0.0, -9.8, 0.0])
    spec = Tri2dSpec(
        V_rest=V, tris=np.concatenate(Ts).astype(np.int32), mu=np.concatenate(mu),
        lam=np.concatenate(lam), V_init=V_init,
        v_init=v_init if np.any(v_init) else None, material=np.concatenate(mat),
        density=None if np.all(rho_all == rho_all[0]) else rho_all,
        density_const=float(rho_all[0]), bc_type=bc[0], bc_axis=bc[1], bc_ratio=bc[2],
        bc_velocity=bc[3], dt=float(args.get("dt", 0.034)),
        body_force=tuple(float(np.float32(v)) for v in bf[:2]),
        bdf_order=_by_name(INTEGRATORS, args.get("time_integrator"), 1),
        max_newton_iterations=int(args.get("max_newton_iterations", 5)),
        max_linesearch_iterations=int(args.get("max_linesearch_iterations", 20)),
        max_iterative_solver_iters=iters, iterative_solver_tolerance=tol,
        linear_solver=solver,
        name=os.path.basename(src) if isinstance(src, str) and not src.lstrip().startswith("{") else "scene")
    for k, v in overrides.items():
        setattr(spec, k, v)
    return spec
