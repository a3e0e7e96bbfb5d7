"""Host-side bookkeeping of the refinement around the largest Berry curvatures (wbgpu.run):
sub-grid shifts and k-point coordinates.  Refining every point of a grid with mesh M gives the
points of the grid with M times more points per axis, shifted by half a sub-cell less than half a
cell."""
import numpy as np

from wbgpu.grid import Grid
from wbgpu.run import block_points, subgrid_shifts


def _grid_points(div, fft, shift=0.0):
    g = Grid(NKdiv=div, NKFFT=fft)
    sh = g.block_shifts() + shift
    nk = int(np.prod(g.FFT))
    return block_points(sh, g.FFT, 1.0 / np.asarray(g.FFT, dtype=float), np.arange(len(sh) * nk)), sh


def _same_set(a, b):
    key = lambda x: np.round(np.mod(x, 1.0) * 1e9).astype(np.int64)
    ka, kb = key(a), key(b)
    return len(ka) == len(kb) and set(map(tuple, ka)) == set(map(tuple, kb))


def test_block_points_cover_the_grid():
    pts, _ = _grid_points((2, 1, 3), (3, 4, 2))
    N = np.array([6, 4, 6])
    ijk = np.stack(np.meshgrid(*[np.arange(n) for n in N], indexing='ij'), -1).reshape(-1, 3)
    assert _same_set(pts, ijk / N)


def test_refine_everything_is_the_finer_grid():
    div, fft, M = (2, 1, 2), (2, 3, 2), 2
    N = np.array(div) * np.array(fft)
    pts, _ = _grid_points(div, fft)
    sub, step = subgrid_shifts(pts, 1.0 / N, M)
    assert np.allclose(step, 1.0 / (N * M))
    fine = block_points(sub, (M, M, M), step, np.arange(len(sub) * M ** 3))
    ref, _ = _grid_points(div, tuple(np.array(fft) * M), shift=-(M - 1) / (2.0 * N * M))
    assert _same_set(fine, ref)
    # a second round of everything: M^2 points per axis, shifted by -(M^2 - 1) / (2 N M^2)
    sub2, step2 = subgrid_shifts(fine, step, M)
    fine2 = block_points(sub2, (M, M, M), step2, np.arange(len(sub2) * M ** 3))
    ref2, _ = _grid_points(div, tuple(np.array(fft) * M * M), shift=-(M * M - 1) / (2.0 * N * M * M))
    assert _same_set(fine2, ref2)
