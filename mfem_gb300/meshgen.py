"""Synthetic cube-grid tetrahedral meshes (5 tets per cube, alternating parity).

Vertex (i, j, k) of an nx*ny*nz grid of cubes has index i + (nx+1)*(j + (ny+1)*k).
Each cube is split into a central tet and four corner tets; the split flips
with the parity of i+j+k so that face diagonals of neighbouring cubes agree.
"""
import numpy as np

# corners as (a, b, c) offsets; central tet + 4 corner tets for even parity
_EVEN = [((0, 0, 0), (1, 1, 0), (1, 0, 1), (0, 1, 1)),
         ((1, 0, 0), (0, 0, 0), (1, 1, 0), (1, 0, 1)),
         ((0, 1, 0), (1, 1, 0), (0, 0, 0), (0, 1, 1)),
         ((0, 0, 1), (1, 0, 1), (0, 1, 1), (0, 0, 0)),
         ((1, 1, 1), (0, 1, 1), (1, 0, 1), (1, 1, 0))]
_ODD = [((1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 1)),
        ((0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1)),
        ((1, 1, 0), (0, 1, 0), (1, 0, 0), (1, 1, 1)),
        ((1, 0, 1), (0, 0, 1), (1, 1, 1), (1, 0, 0)),
        ((0, 1, 1), (1, 1, 1), (0, 0, 1), (0, 1, 0))]


def cube_grid(nx, ny, nz, spacing=0.1, origin=(0.0, 0.0, 0.0)):
    """Returns (V, T): V float64 (nv, 3), T int32 (5*nx*ny*nz, 4), positively oriented."""
    ii, jj, kk = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1),
                             indexing="ij")
    nv = (nx + 1) * (ny + 1) * (nz + 1)
    V = np.empty((nv, 3), dtype=np.float64)
    idx = ii + (nx + 1) * (jj + (ny + 1) * kk)
    V[idx.ravel(), 0] = origin[0] + spacing * ii.ravel()
    V[idx.ravel(), 1] = origin[1] + spacing * jj.ravel()
    V[idx.ravel(), 2] = origin[2] + spacing * kk.ravel()

    ci, cj, ck = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ci, cj, ck = ci.ravel(order="F"), cj.ravel(order="F"), ck.ravel(order="F")
    odd = ((ci + cj + ck) & 1).astype(bool)
    ncube = ci.size
    T = np.empty((ncube, 5, 4), dtype=np.int64)
    for t in range(5):
        for q in range(4):
            ae, be, ce = _EVEN[t][q]
            ao, bo, co = _ODD[t][q]
            a = np.where(odd, ao, ae)
            b = np.where(odd, bo, be)
            c = np.where(odd, co, ce)
            T[:, t, q] = (ci + a) + (nx + 1) * ((cj + b) + (ny + 1) * (ck + c))
    T = T.reshape(-1, 4)
    # orient positively
    X = V[T]
    vol = np.einsum("ij,ij->i", X[:, 1] - X[:, 0], np.cross(X[:, 2] - X[:, 0], X[:, 3] - X[:, 0]))
    neg = vol < 0
    T[neg, 2], T[neg, 3] = T[neg, 3].copy(), T[neg, 2].copy()
    return V, T.astype(np.int32)


def face_mask(V, axis, side="min", tol=None):
    """0/1 int32 mask of vertices on the min or max face of the bounding box along axis."""
    c = V[:, axis]
    lo, hi = c.min(), c.max()
    if tol is None:
        tol = 1e-9 * max(hi - lo, 1.0)
    m = (c <= lo + tol) if side == "min" else (c >= hi - tol)
    return m.astype(np.int32)


def enu_to_lame(E, nu):
    """Enu_to_lame (reference src/config.h:13-16)."""
    E = np.asarray(E, dtype=np.float64)
    nu = np.asarray(nu, dtype=np.float64)
    mu = E / (2.0 * (1.0 + nu))
    lam = (E * nu) / ((1.0 + nu) * (1.0 - 2.0 * nu))
    return lam, mu


def square_grid(nx, ny, spacing=0.1, origin=(0.0, 0.0)):
    """Returns (V, T) of an nx*ny grid of squares in the plane, each split
    into two counter-clockwise triangles along a diagonal that alternates
    with the parity of i+j.  Vertex (i, j) has index i + (nx+1)*j."""
    jj, ii = np.meshgrid(np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    V = np.stack([origin[0] + spacing * ii.ravel(), origin[1] + spacing * jj.ravel()],
                 axis=1).astype(np.float64)
    cj, ci = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    ci, cj = ci.ravel(), cj.ravel()
    v00 = ci + (nx + 1) * cj
    v10, v01, v11 = v00 + 1, v00 + (nx + 1), v00 + nx + 2
    even = ((ci + cj) & 1) == 0
    t1 = np.where(even[:, None], np.stack([v00, v10, v11], 1), np.stack([v00, v10, v01], 1))
    t2 = np.where(even[:, None], np.stack([v00, v11, v01], 1), np.stack([v10, v11, v01], 1))
    T = np.stack([t1, t2], axis=1).reshape(-1, 3)
    return V, T.astype(np.int32)
