"""The stencil predictor's tile skip on the CPU: a 32x8 tile none of whose 3x3 neighbouring tiles
holds a source (a cell with |D| above the threshold, judged by the tiles' maxima as FP32 bit
patterns) has no active cell under the per-cell rule (a source within a diamond of radius 3,
x wrapped on periodic meshes, nothing beyond the mesh in y), and tiles whose reach wraps around a
periodic mesh never skip.  Both rules restated in numpy, as k_conv_next / k_conv_predict apply
them, over ragged tile edges, periodic meshes, sparse fronts and NaN."""
import numpy as np
import pytest

TX, TY, R, ALPHA = 32, 8, 3, np.float32(0.1)


def per_cell_flags(D, solved, thr, periodic):
    Ny, Nx = D.shape
    src = np.abs(D) > thr
    out = np.zeros_like(solved)
    for dj in range(-R, R + 1):
        rx = R - abs(dj)
        for di in range(-rx, rx + 1):
            sh = np.zeros_like(src)
            ys = slice(max(dj, 0), Ny + min(dj, 0))
            yd = slice(max(-dj, 0), Ny + min(-dj, 0))
            if periodic:
                sh[yd, :] = np.roll(src, -di, axis=1)[ys, :]
            else:
                xs = slice(max(di, 0), Nx + min(di, 0))
                xd = slice(max(-di, 0), Nx + min(-di, 0))
                sh[yd, xd] = src[ys, xs]
            out |= sh
    return out & solved


def skipped_tiles(D, thr, periodic):
    Ny, Nx = D.shape
    ntx, nty = -(-Nx // TX), -(-Ny // TY)
    bits = np.abs(D).astype(np.float32).view(np.uint32)
    pad = np.zeros((nty * TY, ntx * TX), np.uint32)
    pad[:Ny, :Nx] = bits
    tmax = pad.reshape(nty, TY, ntx, TX).max(axis=(1, 3)).view(np.float32)
    skip = np.zeros((nty, ntx), bool)
    for by in range(nty):
        for bx in range(ntx):
            i0 = bx * TX
            if periodic and (i0 - R < 0 or i0 + TX - 1 + R >= Nx):
                continue
            near = False
            for ty in range(by - 1, by + 2):
                for tx in range(bx - 1, bx + 2):
                    if 0 <= tx < ntx and 0 <= ty < nty and tmax[ty, tx] > thr:
                        near = True
            skip[by, bx] = not near
    return skip


@pytest.mark.parametrize("Nx,Ny", [(128, 64), (161, 35), (203, 23), (66, 17), (96, 9), (303, 33)])
@pytest.mark.parametrize("periodic", [False, True])
@pytest.mark.parametrize("nan", [False, True])
def test_skipped_tiles_have_no_active_cell(Nx, Ny, periodic, nan):
    rng = np.random.default_rng(Nx * 1000 + Ny + 7 * periodic + 3 * nan)
    for trial in range(6):
        D = (rng.standard_normal((Ny, Nx)) * 1e-9).astype(np.float32)
        # a front: a few columns (and cells near the x edges, which periodic meshes wrap) move much more
        for _ in range(rng.integers(1, 4)):
            c = int(rng.integers(0, Nx))
            D[:, c] += np.float32(1e-4) * rng.standard_normal(Ny).astype(np.float32)
        if trial % 2:
            D[rng.integers(0, Ny), Nx - 1] = np.float32(3e-4)
        if nan and trial == 3:
            D[rng.integers(0, Ny), rng.integers(0, Nx)] = np.float32(np.nan)
        solved = rng.random((Ny, Nx)) > 0.1
        D = np.where(solved, D, np.float32(0))
        gmax = np.abs(D).astype(np.float32).view(np.uint32).max().view(np.float32)
        thr = ALPHA * gmax
        flags = per_cell_flags(D, solved, thr, periodic)
        skip = skipped_tiles(D, thr, periodic)
        ntx, nty = skip.shape[1], skip.shape[0]
        fpad = np.zeros((nty * TY, ntx * TX), bool)
        fpad[:Ny, :Nx] = flags
        active_tiles = fpad.reshape(nty, TY, ntx, TX).any(axis=(1, 3))
        assert not (skip & active_tiles).any(), (trial, np.argwhere(skip & active_tiles))


@pytest.mark.parametrize("periodic", [False, True])
def test_tiles_far_from_a_source_skip(periodic):
    # one source cell in the middle of a 303x33 mesh: only the tiles around it are tested per cell
    Ny, Nx = 33, 303
    D = np.zeros((Ny, Nx), np.float32)
    D[16, 150] = np.float32(1e-4)
    thr = ALPHA * np.float32(1e-4)
    skip = skipped_tiles(D, thr, periodic)
    assert (~skip).sum() == 9 + (2 * skip.shape[0] if periodic else 0)
    assert not per_cell_flags(D, np.ones_like(D, bool), thr, periodic)[:, :100].any()


def test_wrapped_reach_needs_the_per_cell_test():
    # a source in the last column of a periodic mesh activates cells of the first tile column; a
    # skip rule that ignored the wrap (the non-periodic tile neighbourhood) would drop them
    Ny, Nx = 16, 161
    D = np.zeros((Ny, Nx), np.float32)
    D[5, Nx - 1] = np.float32(1e-4)
    thr = ALPHA * np.float32(1e-4)
    flags = per_cell_flags(D, np.ones_like(D, bool), thr, True)
    assert flags[5, 0] and flags[5, 2]
    assert skipped_tiles(D, thr, False)[0, 0]
    assert not skipped_tiles(D, thr, True)[0, 0]
