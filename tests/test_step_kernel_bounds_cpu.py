"""Host-side emulation of the address arithmetic of the precision form's
step kernel (fall3d_gb300/csrc/f3d_fused2.cu, fused2_tile) on grids of many
shapes: every global load and store the kernel makes, under the guard it
makes it under, falls inside its array; 8-byte copies and stores are
8-byte aligned; every tensor copy starts on a 16-byte boundary; and the
shared-memory reads one row beyond a staged field or exchange plane stay
inside the block's allocation.  The tile constants are read from the kernel
source, so the emulation follows them.  compute-sanitizer is not available
to these tests; this is the bounds check that replaces it for this kernel
(the GPU tests then run the kernel on the same kinds of grids)."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = open(os.path.join(ROOT, "fall3d_gb300", "csrc", "f3d_fused2.cu")).read()


def _const(name):
    m = re.search(rf"\b{name} = (\d+)\b", SRC)
    assert m, name
    return int(m.group(1))


HX, HY, NW, GUARD = _const("HX"), _const("HY"), _const("NW"), _const("GUARD")
TX, TY, RS = HX - 6, HY - 6, HX + 4
FS, NP = RS * HY, HX * HY
NF = 9  # F_C .. F_PY of f3d_fused_math.cuh
ZT32_FLOATS = 12


def _positions(nx, ny):
    """Per tile, warp, lane, row r and column c: the tile origin and the
    grid column g and row gj of the position (fused2_tile's i0, j0, gi + c,
    gy0 + 2*warp + r)."""
    tiles_x, tiles_y = -(-nx // TX), -(-ny // TY)
    tile = np.arange(tiles_x * tiles_y)
    i0 = 1 + (tile % tiles_x) * TX
    j0 = 1 + (tile // tiles_x) * TY
    warp = np.arange(NW)
    lane = np.arange(32)
    r = np.arange(HY // NW)
    c = np.arange(2)
    T, W, L, R, Cc = np.meshgrid(tile, warp, lane, r, c, indexing="ij")
    I0, J0 = i0[T], j0[T]
    gx0, gy0 = I0 - 3, J0 - 3
    gi = gx0 + 2 * L
    g = gi + Cc
    gj = gy0 + 2 * W + R
    return dict(I0=I0, J0=J0, gx0=gx0, gy0=gy0, gi=gi, g=g, gj=gj, c=Cc)


def _check(idx, size, what):
    idx = np.asarray(idx)
    assert idx.size == 0 or (idx.min() >= 0 and idx.max() < size), (what, int(idx.min()), int(idx.max()), size)


SHAPES = [(nx, ny, nz) for nx in (3, 4, 5, 57, 58, 59, 60, 63, 64, 116, 117, 175)
          for ny in (3, 4, 25, 26, 27, 53) for nz in (3, 4, 9)]


@pytest.mark.parametrize("nx,ny,nz", SHAPES)
def test_global_accesses_stay_in_their_arrays(nx, ny, nz):
    p = _positions(nx, ny)
    g, gj, gi, c = p["g"], p["gj"], p["gi"], p["c"]
    I0, J0 = p["I0"], p["J0"]
    px, pl = nx + 2, nx * ny
    cs = px * (ny + 2)
    csize = cs * (nz + 2)  # one class of c
    hp = (nx + 2 + 3) & ~3  # halo_pitch
    hs = hp * (ny + 2)
    hsize = hs * (nz + 2)  # one met field (or one class of vz+vset) in the halo layout
    p8 = nx % 2 == 0
    kin = (g >= 1) & (g <= nx) & (gj >= 1) & (gj <= ny)
    inr = (g >= 0) & (g <= nx + 1) & (gj >= 0) & (gj <= ny + 1)
    oi1, oj1 = np.minimum(nx, I0 + TX - 1), np.minimum(ny, J0 + TY - 1)
    out = kin & (g >= I0) & (g <= oi1) & (gj >= J0) & (gj <= oj1)

    # bottom ghost window: c planes 1 and 2, vz+vset plane 1, the 2-D fields
    hb = (g + px * gj)[kin]
    _check(hb + cs, csize, "c plane 1")
    _check(hb + 2 * cs, csize, "c plane 2")
    _check((g + hp * gj + hs)[kin], hsize, "vz+vset plane 1")
    mb = ((g - 1) + nx * (gj - 1))[kin]
    _check(mb, pl, "vdep / rkver / zi / lambda")

    # staged c of plane t+2 (t + 2 <= nz): a pair's offset from its first
    # column, clamped to plane 1 for pairs outside the halo array
    inr0 = inr[..., 0]
    h0 = np.where(inr0, gi[..., 0] + px * gj[..., 0], cs)
    for t in range(1, nz - 1):
        off = h0 + (t + 2) * cs
        _check(off, csize, "c copy address")
        if p8:
            _check(off[inr0], csize - 1, "c 8-byte copy")
            assert np.all(off[inr0] % 2 == 0), "8-byte copy not aligned"
        else:
            _check(off[inr[..., 1]] + 1, csize, "c second column copy")

    # y-face ghosts of plane t <= nz: the adjacent row's c and vy
    yg = ((gj == 0) | (gj == ny + 1)) & (g >= 1) & (g <= nx)
    ja = np.where(gj == 0, 1, ny)
    for t in (1, nz):
        _check((g + px * ja + t * cs)[yg], csize, "y ghost c")
        _check((g + hp * ja + t * hs)[yg], hsize, "y ghost vy")

    # diffz's last plane: 1/rho and K*rho at nz-1 of every position in the array
    _check((g + hp * gj + (nz - 1) * hs)[inr], hsize, "1/rho, K*rho plane nz-1")

    # stores: output cells at planes 1..nz, the outer ghosts, planes 0 and nz+1
    for k in (0, 1, nz, nz + 1):
        _check((g + px * gj + k * cs)[out], csize, f"store plane {k}")
    kgx = ((g == 0) | (g == nx + 1)) & (gj >= 1) & (gj <= ny)
    kgy = ((gj == 0) | (gj == ny + 1)) & (g >= 1) & (g <= nx)
    rows_out, cols_out = (gj >= J0) & (gj <= oj1), (g >= I0) & (g <= oi1)
    ghost_st = (kgx & rows_out & (((g == 0) & (I0 == 1)) | ((g == nx + 1) & (oi1 == nx)))) | \
               (kgy & cols_out & (((gj == 0) & (J0 == 1)) | ((gj == ny + 1) & (oj1 == ny))))
    for k in (1, nz):
        _check((g + px * gj + k * cs)[ghost_st], csize, "outer ghost store")
    if p8:  # a pair stored as one 8-byte value only when both columns store
        both = (out | ghost_st).all(axis=-1)
        assert np.all((gi[..., 0] + px * gj[..., 0])[both] % 2 == 0) and cs % 2 == 0

    # every output cell of the grid is written by exactly one tile
    cells = ((g - 1) + nx * (gj - 1))[out]
    assert np.array_equal(np.sort(cells), np.arange(pl)), "output tiles do not cover the grid once"

    # tensor copies: boxes of RS x HY from the region's first column rounded
    # down to a multiple of 4 floats (16 bytes), covering the region
    xs = p["gx0"] & ~3
    assert np.all(xs % 4 == 0)
    assert np.all((p["gx0"] - xs >= 0) & (p["gx0"] - xs + HX <= RS))


def test_shared_memory_reads_stay_in_the_block():
    """fused_tile's shared layout: GUARD bytes, the two staging buffers of
    NF fields, the P0 / W1 / W2 / P1 planes (the last with HX floats of
    padding), the wet accumulators and the plane table.  The reads one row
    above a warp's pair (row -1 of warp 0) and one or two rows below it
    (rows 32, 33 of warp 15) must stay inside that allocation."""
    nz = 80
    smem = 128 + GUARD + 4 * (2 * NF * FS + 4 * NP + HX) + (2 * 8 + 4) * TX * TY + 4 * ZT32_FLOATS * (nz + 1) + 32
    # offsets in floats from the start of the staging area (after the GUARD)
    lo, hi = -GUARD // 4, (smem - 128 - GUARD) // 4
    lanes, warps = np.arange(32), np.arange(NW)
    W, L = np.meshgrid(warps, lanes, indexing="ij")
    for sft in (0, 2):
        for buf in (0, 1):
            row0 = buf * NF * FS + 2 * W * RS + sft + 2 * L
            for field in range(NF):
                base = row0 + field * FS
                for off in (-RS, 0, RS, 2 * RS):  # rows -1..2 around the pair
                    idx = base + off
                    assert idx.min() >= lo and idx.max() + 1 < hi
    p0 = 2 * NF * FS
    for plane in range(4):  # P0s, W1s, W2s, P1s
        base = p0 + plane * NP + 2 * W * HX + 2 * L
        for off in (-HX, 0, HX, 2 * HX):
            idx = base + off
            assert idx.min() >= lo and idx.max() + 1 < p0 + 4 * NP + HX
