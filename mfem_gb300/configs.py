"""The benchmark workloads as scene specs (synthetic cube-grid meshes).

  beam_c1     3-D beam 10x2x2 cubes of 0.1 m, 5 tets/cube (200 tets, 99 vertices),
              stable neo-Hookean E=1e6 Pa, nu=0.45, rho=1000; x=0 face pinned;
              BDF1 dt=1/60; gravity; <=10 Newton iterations; PCG tol 1e-8; FP64.
  cube_c2     60^3 cubes at 0.01 m (1.08M tets, 226,981 vertices), E=1e5, nu=0.45,
              vertex positions perturbed i.i.d. U(+-10% of the spacing) (a jittered
              mesh, starting at rest); bottom layer pinned; BDF1 dt=1/60; FP32
              element work + FP64 reductions.
  stress_c3   30^3 cubes (135k tets), nu=0.495, per-tet E log-uniform in [1e4, 1e7];
              the x-max face compresses 50% along x over 20 steps, x-min face pinned;
              dt=1/100; Newton to 1e-5 relative residual.
  batch_c4    64 scenes, nx, ny, nz ~ U{4..30}, E log-U[1e4, 1e6], nu U[0.3, 0.48],
              one random face pinned, gravity, dt=1/60.
  stream_c5   Poisson arrivals of scenes with tet counts log-U[1e3, 5e5].
"""
import math

import numpy as np

from . import abi
from .desc import SceneSpec
from .meshgen import cube_grid, enu_to_lame, face_mask

SEED = 20261203


def beam_c1(precision=abi.PRECISION_FP64, **kw):
    V, T = cube_grid(10, 2, 2, 0.1)
    lam, mu = enu_to_lame(1e6, 0.45)
    spec = SceneSpec(V_rest=V, tets=T, mu=np.full(len(T), mu), lam=np.full(len(T), lam),
                     is_fixed=face_mask(V, 0, "min"), density_const=1000.0, dt=1.0 / 60.0,
                     body_force=(0.0, -9.8, 0.0), max_newton_iterations=10,
                     iterative_solver_tolerance=1e-8, max_iterative_solver_iters=500,
                     precision=precision, name="beam_c1")
    for k, v in kw.items():
        setattr(spec, k, v)
    return spec


def cube_c2(n=60, spacing=0.01, precision=abi.PRECISION_MIXED, seed=SEED, perturb_initial_only=False,
            **kw):
    """By default the vertex perturbation jitters the mesh: rest and initial
    positions are the perturbed grid, so the body starts undeformed and sags
    under gravity from its pinned bottom layer (j = 0 of the grid).  With
    perturb_initial_only the rest mesh is the regular grid and only the
    initial positions are perturbed, so the body starts pre-strained."""
    V, T = cube_grid(n, n, n, spacing)
    pinned = face_mask(V, 1, "min")
    rng = np.random.default_rng(seed)
    Vp = V + rng.uniform(-0.1 * spacing, 0.1 * spacing, size=V.shape)
    V_init = None
    if perturb_initial_only:
        V_init = Vp
    else:
        V = Vp
    lam, mu = enu_to_lame(1e5, 0.45)
    spec = SceneSpec(V_rest=V, tets=T, mu=np.full(len(T), mu), lam=np.full(len(T), lam), V_init=V_init,
                     is_fixed=pinned, density_const=1000.0, dt=1.0 / 60.0,
                     body_force=(0.0, -9.8, 0.0), max_newton_iterations=40,
                     iterative_solver_tolerance=1e-4, max_iterative_solver_iters=500,
                     newton_residual_tolerance=1e-5, precision=precision, name=f"cube_c2_{n}")
    for k, v in kw.items():
        setattr(spec, k, v)
    return spec


def stress_c3(n=30, spacing=0.01, precision=abi.PRECISION_MIXED, seed=SEED, steps=20, **kw):
    V, T = cube_grid(n, n, n, spacing)
    rng = np.random.default_rng(seed + 3)
    E = np.exp(rng.uniform(math.log(1e4), math.log(1e7), size=len(T)))
    lam, mu = enu_to_lame(E, 0.495)
    dt = 1.0 / 100.0
    length = n * spacing
    spec = SceneSpec(V_rest=V, tets=T, mu=mu, lam=lam, density_const=1000.0, dt=dt,
                     body_force=(0.0, -9.8, 0.0), bc_type=abi.BC_COMPRESS, bc_axis=0,
                     bc_ratio=0.5 / n, bc_velocity=-0.5 * length / (steps * dt),
                     max_newton_iterations=20, iterative_solver_tolerance=1e-4,
                     max_iterative_solver_iters=1000, newton_residual_tolerance=1e-5,
                     precision=precision, name=f"stress_c3_{n}")
    for k, v in kw.items():
        setattr(spec, k, v)
    return spec


def random_scene(rng, dims, precision=abi.PRECISION_MIXED, spacing=0.01, **kw):
    nx, ny, nz = dims
    V, T = cube_grid(nx, ny, nz, spacing)
    E = math.exp(rng.uniform(math.log(1e4), math.log(1e6)))
    nu = rng.uniform(0.3, 0.48)
    lam, mu = enu_to_lame(E, nu)
    axis = int(rng.integers(0, 3))
    side = "min" if rng.integers(0, 2) == 0 else "max"
    spec = SceneSpec(V_rest=V, tets=T, mu=np.full(len(T), float(mu)), lam=np.full(len(T), float(lam)),
                     is_fixed=face_mask(V, axis, side), density_const=1000.0, dt=1.0 / 60.0,
                     body_force=(0.0, -9.8, 0.0), max_newton_iterations=10,
                     iterative_solver_tolerance=1e-4, max_iterative_solver_iters=500,
                     newton_residual_tolerance=1e-5, precision=precision,
                     name=f"grid_{nx}x{ny}x{nz}")
    for k, v in kw.items():
        setattr(spec, k, v)
    return spec


def batch_c4(count=64, seed=SEED, precision=abi.PRECISION_MIXED, lo=4, hi=30, **kw):
    rng = np.random.default_rng(seed + 4)
    specs = []
    for _ in range(count):
        dims = tuple(int(v) for v in rng.integers(lo, hi + 1, size=3))
        specs.append(random_scene(rng, dims, precision=precision, **kw))
    return specs


def stream_c5(rate=20.0, duration=60.0, seed=SEED, tet_lo=1e3, tet_hi=5e5, steps=200,
              precision=abi.PRECISION_MIXED):
    """Yields (arrival_time_s, spec, steps) for Poisson arrivals."""
    rng = np.random.default_rng(seed + 5)
    t = 0.0
    out = []
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        tets = math.exp(rng.uniform(math.log(tet_lo), math.log(tet_hi)))
        cubes = max(1.0, tets / 5.0)
        a = rng.uniform(1.0, 4.0, size=3)
        scale = (cubes / np.prod(a)) ** (1.0 / 3.0)
        dims = tuple(max(1, int(round(v * scale))) for v in a)
        out.append((t, random_scene(rng, dims, precision=precision), steps))
    return out
