"""The segmented line solve of the mixed path (k_sweep_seg), restated in
numpy: segmentation rule, row tables and carries, checked against the
sequential LU solve (src/Subroutines3D.f90:124-136) on banded systems of the
compact scheme's shape.  The GPU path itself is checked against the FP64
engine in test_mixed_gpu.py; this pins the algebra and the index rules the
kernel and the host tables share."""
import re
from pathlib import Path

import numpy as np
import pytest

HDR = Path(__file__).resolve().parents[1] / "tandemproject_gb300" / "csrc" / "ati_kernels.h"


def constants():
    txt = HDR.read_text()
    m = re.search(r"constexpr int SEG_LINES = (\d+), SEG_ROWS = (\d+), SEG_MAX = (\d+), SEG_LMAX = (\d+);", txt)
    assert m, "segment constants not found in ati_kernels.h"
    return tuple(int(v) for v in m.groups())


SEG_LINES, SEG_ROWS, SEG_MAX, SEG_LMAX = constants()


def seg_count(L):
    return max(1, min(SEG_MAX, (L + SEG_ROWS - 1) // SEG_ROWS))


def seg_start(k, L, S):
    q, r = divmod(L, S)
    return k * q + min(k, r)


def banded(L, rng):
    """A diagonally dominant pentadiagonal matrix and its LU factors in the
    layout of the solver's factor table: per row l0, l1 (sub-diagonals of L),
    c2 = 1/u_ii, c3, c4 (super-diagonals of U over u_ii); entries a row does
    not have are set to 1, as the table holds them."""
    A = np.zeros((L, L))
    for i in range(L):
        A[i, i] = 1.0
        for o, c in ((-2, 0.0955), (-1, 0.5863), (1, 0.5863), (2, 0.0955)):
            if 0 <= i + o < L:
                A[i, i + o] = c * (1 + 0.05 * rng.standard_normal())
    U = A.copy()
    Lm = np.eye(L)
    for k in range(L):
        for i in range(k + 1, min(k + 3, L)):
            m = U[i, k] / U[k, k]
            Lm[i, k] = m
            U[i, :] -= m * U[k, :]
    fac = np.ones((L, 5))
    for i in range(L):
        if i >= 2:
            fac[i, 0] = Lm[i, i - 2]
        if i >= 1:
            fac[i, 1] = Lm[i, i - 1]
        fac[i, 2] = 1 / U[i, i]
        if i + 1 < L:
            fac[i, 3] = U[i, i + 1] / U[i, i]
        if i + 2 < L:
            fac[i, 4] = U[i, i + 2] / U[i, i]
    return A, fac


def sequential(fac, r, dtype=np.float64):
    fac = fac.astype(dtype)
    L = len(r)
    r = r.astype(dtype)
    v = np.zeros(L, dtype)
    for i in range(L):
        v[i] = r[i] - (fac[i, 0] * v[i - 2] if i >= 2 else 0) - (fac[i, 1] * v[i - 1] if i >= 1 else 0)
    b = np.zeros(L, dtype)
    for i in range(L - 1, -1, -1):
        b[i] = fac[i, 2] * v[i] - (fac[i, 3] * b[i + 1] if i <= L - 2 else 0) - (fac[i, 4] * b[i + 2] if i <= L - 3 else 0)
    return b


def row_table(fac):
    """The host's row table (ati_api.cu seg_tables): masked factors and the
    forward (g, h) and backward (G, H) responses of each row's segment."""
    L = len(fac)
    S = seg_count(L)
    t = np.zeros((L, 12))
    t[:, 0] = [fac[i, 0] if i >= 2 else 0 for i in range(L)]
    t[:, 1] = [fac[i, 1] if i >= 1 else 0 for i in range(L)]
    t[:, 6] = fac[:, 2]
    t[:, 7] = [fac[i, 3] if i <= L - 2 else 0 for i in range(L)]
    t[:, 10] = [fac[i, 4] if i <= L - 3 else 0 for i in range(L)]
    for k in range(S):
        s0, s1 = seg_start(k, L, S), seg_start(k + 1, L, S)
        if k > 0:
            g2, g1, h2, h1 = 1.0, 0.0, 0.0, 1.0
            for i in range(s0, s1):
                g = -t[i, 0] * g2 - t[i, 1] * g1
                h = -t[i, 0] * h2 - t[i, 1] * h1
                t[i, 4], t[i, 5] = g, h
                g2, g1, h2, h1 = g1, g, h1, h
        if k < S - 1:
            G1, G2, H1, H2 = 1.0, 0.0, 0.0, 1.0
            for i in range(s1 - 1, s0 - 1, -1):
                G = -t[i, 7] * G1 - t[i, 10] * G2
                H = -t[i, 7] * H1 - t[i, 10] * H2
                t[i, 8], t[i, 9] = G, H
                G2, G1, H2, H1 = G1, G, H1, H
    return t


def segmented(t, r, dtype=np.float64):
    """The kernel's phases 3-7 for one line (right-hand side r given)."""
    t = t.astype(dtype)
    L = len(r)
    S = seg_count(L)
    col = r.astype(dtype).copy()
    cf = np.zeros((S, 2), dtype)
    cx = np.zeros((S, 2), dtype)
    for w in range(S):  # forward, zero incoming values
        s0, s1 = seg_start(w, L, S), seg_start(w + 1, L, S)
        pm2 = pm1 = dtype(0)
        for i in range(s0, s1):
            p = col[i] - t[i, 0] * pm2 - t[i, 1] * pm1
            col[i] = p
            pm2, pm1 = pm1, p
        cf[w] = (pm2, pm1)
    x = np.zeros(2, dtype)
    for k in range(1, S):  # forward carry
        e = seg_start(k, L, S)
        c = cf[k - 1]
        x = np.array([c[0] + t[e - 2, 4] * x[0] + t[e - 2, 5] * x[1], c[1] + t[e - 1, 4] * x[0] + t[e - 1, 5] * x[1]])
        cx[k] = x
    for w in range(S):  # correction, back substitution from zero values beyond the segment
        s0, s1 = seg_start(w, L, S), seg_start(w + 1, L, S)
        q1 = q2 = dtype(0)
        for i in range(s1 - 1, s0 - 1, -1):
            v = col[i] + t[i, 4] * cx[w, 0] + t[i, 5] * cx[w, 1]
            q = t[i, 6] * v - t[i, 7] * q1 - t[i, 10] * q2
            col[i] = q
            q2, q1 = q1, q
        cf[w] = (q1, q2)
    cx[:] = 0
    y = np.zeros(2, dtype)
    for k in range(S - 2, -1, -1):  # backward carry
        e = seg_start(k + 1, L, S)
        c = cf[k + 1]
        y = np.array([c[0] + t[e, 8] * y[0] + t[e, 9] * y[1], c[1] + t[e + 1, 8] * y[0] + t[e + 1, 9] * y[1]])
        cx[k] = y
    out = np.zeros(L, dtype)
    for w in range(S):
        s0, s1 = seg_start(w, L, S), seg_start(w + 1, L, S)
        for i in range(s0, s1):
            out[i] = col[i] + t[i, 8] * cx[w, 0] + t[i, 9] * cx[w, 1]
    return out


@pytest.mark.parametrize("L", [13, 24, 32, 48, 49, 96, 120, 121, 256, 384, 640, 1000, SEG_LMAX])
def test_segmented_solve_matches_sequential(L):
    rng = np.random.default_rng(L)
    A, fac = banded(L, rng)
    t = row_table(fac)
    for _ in range(2):
        r = rng.standard_normal(L)
        bs = sequential(fac, r)
        assert np.max(np.abs(bs - np.linalg.solve(A, r))) < 1e-11 * np.max(np.abs(bs))
        bg = segmented(t, r)
        assert np.max(np.abs(bg - bs)) < 1e-12 * np.max(np.abs(bs))
        # in FP32 (the mixed path's arithmetic) the segmented order is as accurate as the sequential one
        # (the derivative matrix is nearly singular at the grid's odd-even mode, so both lose some digits)
        e_seg = np.max(np.abs(segmented(t, r, np.float32) - bs))
        e_seq = np.max(np.abs(sequential(fac, r, np.float32) - bs))
        assert e_seg < 4 * e_seq + 1e-6 * np.max(np.abs(bs)), (e_seg, e_seq)


@pytest.mark.parametrize("L", list(range(13, 200)) + [383, 384, 385, 639, 640, 1599, SEG_LMAX])
def test_segment_rules(L):
    """Every segment is long enough for the kernel's windows (at least 12
    rows, so the three rows after it, its first window and the carry rows lie
    where the kernel reads them) and the tile fits the shared memory."""
    S = seg_count(L)
    bounds = [seg_start(k, L, S) for k in range(S + 1)]
    assert bounds[0] == 0 and bounds[-1] == L
    assert all(b - a >= 12 for a, b in zip(bounds, bounds[1:])), bounds
    assert max(b - a for a, b in zip(bounds, bounds[1:])) - min(b - a for a, b in zip(bounds, bounds[1:])) <= 1
    smem = S * SEG_LINES * 16 + L * (SEG_LINES + 1) * 4
    assert smem <= 227 * 1024
    assert S * SEG_LINES <= SEG_LINES * SEG_MAX
    if S == 1:  # one-segment lines: SEG_GROUPS groups of lines share a CTA, each with its own tile
        groups = int(re.search(r"constexpr int SEG_GROUPS = (\d+);", HDR.read_text()).group(1))
        assert groups * SEG_LINES * 16 + groups * L * (SEG_LINES + 1) * 4 <= 227 * 1024
        assert groups * SEG_LINES <= SEG_LINES * SEG_MAX
