"""FP64 reference solve of the world step's pressure problem.

Test infrastructure: the tests call it to check the mixed-precision
pressure solve; the library and the benchmark never do.

The operator is the level-0 operator of the reference's multigrid
(shaders/world/multigrid.wgsl:29-77: the Gauss-Seidel update
p = (sum over water neighbours of p_j - rhs) / (k + eps) solves
L p = rhs with L p = sum_j p_j - (k + eps) p on water cells), written as
    (L p)_i = sum over water neighbours j of (p_j - p_i) - eps0 * p_i
with eps0 the f32 value of 1e-4 (src/world/mod.rs:637-671, MG_EPS), exact in
FP64.  Wall cells are not unknowns.
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spl

EPS0 = float(np.float32(1e-4))


def operator(water: np.ndarray):
    """(L as a CSR matrix over the water cells, flat indices of the water cells)."""
    h, w = water.shape
    flat = water.reshape(-1)
    cells = np.nonzero(flat)[0]
    pos = -np.ones(h * w, np.int64)
    pos[cells] = np.arange(cells.size)
    idx = np.arange(h * w).reshape(h, w)
    rows, cols = [], []
    k = np.zeros(h * w)
    for dy, dx in ((0, 1), (0, -1), (1, 0), (-1, 0)):
        y0, y1 = max(0, -dy), h - max(0, dy)
        x0, x1 = max(0, -dx), w - max(0, dx)
        src = idx[y0:y1, x0:x1].reshape(-1)
        dst = idx[y0 + dy:y1 + dy, x0 + dx:x1 + dx].reshape(-1)
        m = flat[src] & flat[dst]
        rows.append(pos[src[m]])
        cols.append(pos[dst[m]])
        np.add.at(k, src[m], 1.0)
    rows = np.concatenate(rows)
    cols = np.concatenate(cols)
    n = cells.size
    off = sp.coo_matrix((np.ones(rows.size), (rows, cols)), shape=(n, n)).tocsr()
    return (off - sp.diags(k[cells] + EPS0)).tocsr(), cells


def apply(p: np.ndarray, water: np.ndarray) -> np.ndarray:
    """L p on the water cells (0 on walls), in FP64, from a field p."""
    p = np.where(water, np.asarray(p, np.float64), 0.0)
    s = np.zeros_like(p)
    s[:, 1:] += np.where(water[:, :-1] & water[:, 1:], p[:, :-1] - p[:, 1:], 0.0)
    s[:, :-1] += np.where(water[:, 1:] & water[:, :-1], p[:, 1:] - p[:, :-1], 0.0)
    s[1:, :] += np.where(water[:-1, :] & water[1:, :], p[:-1, :] - p[1:, :], 0.0)
    s[:-1, :] += np.where(water[1:, :] & water[:-1, :], p[1:, :] - p[:-1, :], 0.0)
    return np.where(water, s - EPS0 * p, 0.0)


def rel_residual(p: np.ndarray, rhs: np.ndarray, water: np.ndarray) -> float:
    """||rhs - L p|| / ||rhs|| over the water cells, in FP64."""
    b = np.where(water, np.asarray(rhs, np.float64), 0.0)
    bn = np.linalg.norm(b)
    return float(np.linalg.norm(b - apply(p, water)) / bn) if bn > 0 else 0.0


def solve(rhs: np.ndarray, water: np.ndarray) -> np.ndarray:
    """The exact FP64 solution of L p = rhs (sparse direct), 0 on walls."""
    A, cells = operator(water)
    x = spl.spsolve(A.tocsc(), np.asarray(rhs, np.float64).reshape(-1)[cells])
    p = np.zeros(water.size)
    p[cells] = x
    return p.reshape(water.shape)
