"""Generate tests/golden/line_operators.npz: an independent numpy restatement
of the reference's compact line operators, used to pin the C oracle.

The reference ships no tests or recorded outputs and cannot be compiled here,
so these fixtures are derived from its source formulas by a second, separate
implementation:
  * sbcco (src/Subroutineso.f90:107-159) built with numpy.linalg.inv instead
    of the Gauss-Jordan mtrxi,
  * fcint/fcbcm filter coefficients (src/Subroutineso.f90:71-103),
  * deriv and filte (src/Subroutines3D.f90:84-206) as dense matrices: the
    right-hand-side rows (including the periodic closure of mpigo with a
    self exchange, src/Subroutines3D.f90:16-80) evaluated on unit vectors,
    and the pentadiagonal left-hand side (src/Main3D.f90:295-307) solved with
    numpy.linalg.solve instead of the LU recurrence of penta.

Run:  python tests/golden/make_golden.py   (writes line_operators.npz)
"""
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LMD, LMF = 11, 8
alpha, beta = 0.5862704032801503, 0.09549533555017055
aa, ab, ac = 0.6431406736919156, 0.2586011023495066, 0.007140953479797375
beta20, alpha21, alpha23, beta24 = 0.03250008295108466, 0.3998040493524358, 0.7719261277615860, 0.1626635931256900
a2 = [-0.1219006056449124, -0.6301651351188667, 0.6521195063966084, 0.3938843551210350, 0.01904944407973912,
      -0.001027260523947668]
alpha10, alpha12, beta13 = 0.08360703307833438, 2.058102869495757, 0.9704052014790193
a1 = [-0.3177447290722621, -0.02807631929593225, 1.593461635747659, 0.2533027046976367, -0.03619652460174756,
      0.004080281419108407]
alpha01, beta02 = 5.912678614078549, 3.775623951744012
a0 = [-3.456878182643609, 5.839043358834730, 1.015886726041007, -0.2246526470654333, 0.08564940889936562,
      -0.01836710059356763]
ABC = np.array([a0, a1, a2])  # abc(:,r)
ALBED = {0: [[0, 0, 1, alpha01, beta02], [0, alpha10, 1, alpha12, beta13], [beta20, alpha21, 1, alpha23, beta24]],
         1: [[0, 0, 1, alpha, beta], [0, alpha, 1, alpha, beta], [beta, alpha, 1, alpha, beta]]}


def fcint(fltk, fltr):
    c1, c2, c3 = math.cos(fltk), math.cos(2 * fltk), math.cos(3 * fltk)
    f = 1 / (30 + 5 * (7 - 16 * fltr) * c1 + 2 * (1 + 8 * fltr) * c2 - 3 * c3)
    al = f * (20 * (2 * fltr - 1) - 30 * c1 + 12 * (2 * fltr - 1) * c2 - 2 * c3)
    be = 0.5 * f * (2 * (13 - 8 * fltr) + (33 - 48 * fltr) * c1 + 6 * c2 - c3)
    za = 60 * (1 - fltr) * math.cos(0.5 * fltk) ** 4 * f
    return al, be, za, -2 * za / 5, za / 15


def filter_rows(fltk, fltkbc):
    res = (fltkbc - fltk) / 9
    out = []
    for i, kk in enumerate((fltk + 9 * res, fltk + 4 * res, fltk + res)):
        al, be, za, zb, zc = fcint(kk, 0.5)
        if i == 0:
            f = 1 / (1 + al / 2 + be / 4)
            out.append(([0, 0, 1, al * f, be * f], za * f, zb * f, zc * f))
        elif i == 1:
            out.append(([0, al + be / 2, 1, al, be], za, zb, zc))
        else:
            out.append(([be, al, 1, al, be], za, zb, zc))
    return out


def sbcco(fltk):
    pbci = np.zeros((2, 2, 12))
    pbco = np.zeros((2, 2, 12))
    for nt in (0, 1):
        lp = 2 * nt - 1
        ll = LMD if nt == 0 else LMF
        n = 2 * (ll + 1)
        ax = np.zeros((n, n))
        bx = np.zeros((n, n))
        if nt == 0:
            s = ABC.sum(axis=1)
            ax[0, 0:3] = ALBED[0][0][2:5]
            ax[1, 0:4] = ALBED[0][1][1:5]
            ax[2, 0:5] = ALBED[0][2]
            bx[0, 0:7] = [-s[0]] + a0
            bx[1, 0:7] = [a1[0], -s[1]] + a1[1:]
            bx[2, 0:7] = [a2[0], a2[1], -s[2]] + a2[2:]
            for i in range(3, n - 3):
                ax[i, i - 2:i + 3] = [beta, alpha, 1, alpha, beta]
                bx[i, i - 3:i + 4] = [-ac, -ab, -aa, 0, aa, ab, ac]
        else:
            al, be, za, zb, zc = fcint(fltk, 0.5)
            zv = [zb + 5 * zc, za - 10 * zc, za - 5 * zc, zb + zc, zc]
            f = 1 / (1 + 5 * al ** 3 + al ** 2 * (8 + 22 * be) + be * (5 + 4 * be + 60 * be ** 2)
                     + 5 * al * (1 + be * (3 + 10 * be)))
            r0 = (al * (1 + al) * (1 + 4 * al) + 2 * al * (7 + 3 * al) * be + 24 * (1 - al) * be ** 2
                  - 80 * be ** 3) * f
            r1 = (al ** 3 + be + 14 * al ** 2 * be + 60 * be ** 3 + al * be * (3 + 46 * be)) * f
            ax[0, 0:3] = [1, r0, r1]
            f = 1 / (1 + al ** 2 * (9 - 5 * be) + al * (5 + (35 - 29 * be) * be) + be * (5 + 6 * (9 - 10 * be) * be))
            r0 = (9 * al ** 3 + 10 * be ** 2 * (8 * be - 1) + 5 * al ** 2 * (1 + 8 * be)
                  + al * (1 + be * (4 + 81 * be))) * f
            r1 = (al * (1 + al * (5 + 9 * al)) + al * (5 + 36 * al) * be + (55 * al - 1) * be ** 2
                  + 10 * be ** 3) * f
            r2 = be * (1 + al * (5 + 9 * al) + 5 * be + 35 * al * be + 50 * be ** 2) * f
            ax[1, 0:4] = [r0, 1, r1, r2]
            ax[2, 0:5] = [be, al, 1, al, be]
            bx[2, 0:6] = [zv[0], zv[1], -sum(zv), zv[2], zv[3], zv[4]]
            for i in range(3, n - 3):
                ax[i, i - 2:i + 3] = [be, al, 1, al, be]
                bx[i, i - 3:i + 4] = [zc, zb, za, -2 * (za + zb + zc), za, zb, zc]
        for r in range(3):
            ax[n - 1 - r, ::-1] = ax[r, :]
            bx[n - 1 - r, ::-1] = lp * bx[r, :]
        sx = np.linalg.inv(ax)
        rx = ax.copy()
        i = n // 2 - 2
        rx[i, i + 2] = 0; rx[i + 1, i + 2] = 0; rx[i + 1, i + 3] = 0
        i = n // 2 + 1
        rx[i, i - 2] = 0; rx[i - 1, i - 2] = 0; rx[i - 1, i - 3] = 0
        cx = rx @ (sx @ bx)
        for j in (0, 1):
            row = n // 2 + j
            pbco[nt, j, :ll + 1] = cx[row, 0:ll + 1][::-1]
            pbci[nt, j, :ll + 1] = cx[row, ll + 1:n]
    return pbci, pbco


def lhs(L, rows_s, rows_e, al, be):
    A = np.zeros((L, L))
    for i in range(L):
        if i < 3:
            row = rows_s[i]
            for o in range(-2, 3):
                if 0 <= i + o < L:
                    A[i, i + o] = row[o + 2]
        elif i > L - 4:
            row = rows_e[L - 1 - i]
            for o in range(-2, 3):
                if 0 <= i - o < L:
                    A[i, i - o] = row[o + 2]
        else:
            A[i, i - 2:i + 3] = [be, al, 1, al, be]
    return A


def deriv_rhs(f, periodic, pbci, pbco):
    """RHS of deriv for one line; periodic = BC 45 at both ends (self exchange
    through mpigo with n45 = 0: recv of one end = send of the other)."""
    L = len(f)
    sb = np.zeros(L)
    if not periodic:
        o = [[1, 2, 3, 4, 5, 6], [0, 2, 3, 4, 5, 6], [0, 1, 3, 4, 5, 6]]
        for r in range(3):
            sb[r] = sum(ABC[r, q] * (f[o[r][q]] - f[r]) for q in range(6))
            sb[L - 1 - r] = sum(ABC[r, q] * (f[L - 1 - r] - f[L - 1 - o[r][q]]) for q in range(6))
    else:
        def send(ip):  # ii = 1 skips the shared end point
            sap = [f[L - 1 - (i + 1)] if ip == 1 else f[i + 1] for i in range(LMD + 1)]
            return (sum(pbco[0, 0, i] * sap[i] for i in range(LMD + 1)),
                    sum(pbco[0, 1, i] * sap[i] for i in range(LMD + 1)), sap[0])
        r0 = send(1)  # recv(:,:,0) comes from face 1
        r1 = send(0)
        sb[0] = sum(pbci[0, 0, q] * f[q] for q in range(LMD + 1)) + r0[0]
        sb[1] = sum(pbci[0, 1, q] * f[q] for q in range(LMD + 1)) + r0[1]
        sb[2] = aa * (f[3] - f[1]) + ab * (f[4] - f[0]) + ac * (f[5] - r0[2])
        sb[L - 1] = -sum(pbci[0, 0, q] * f[L - 1 - q] for q in range(LMD + 1)) - r1[0]
        sb[L - 2] = -sum(pbci[0, 1, q] * f[L - 1 - q] for q in range(LMD + 1)) - r1[1]
        sb[L - 3] = aa * (f[L - 2] - f[L - 4]) + ab * (f[L - 1] - f[L - 5]) + ac * (r1[2] - f[L - 6])
    for i in range(3, L - 3):
        sb[i] = aa * (f[i + 1] - f[i - 1]) + ab * (f[i + 2] - f[i - 2]) + ac * (f[i + 3] - f[i - 3])
    return sb


def filter_rhs(f, periodic, pbci, pbco, frows, fint):
    L = len(f)
    fa, fb, fc = fint
    fam = [r[1] for r in frows]; fbm = [r[2] for r in frows]; fcm = [r[3] for r in frows]
    fex = [45 / 30.0, -9 / 30.0, 1 / 30.0]
    ffx = [4 / (8 * math.log(2.0)), 6 / (8 * math.log(2.0)), 7 / (8 * math.log(2.0))]
    sb = np.zeros(L)
    if not periodic:
        for side in (0, 1):
            g = f if side == 0 else f[::-1]
            res = sum(fex[q] * (g[q + 1] - g[0]) for q in range(3))
            rv = [g[0] - res * ffx[q] for q in range(3)]
            r0, r1, r2 = 2 * g[0], 2 * g[1], 2 * g[2]
            s0 = fam[0] * (rv[0] + g[1] - r0) + fbm[0] * (rv[1] + g[2] - r0) + fcm[0] * (rv[2] + g[3] - r0)
            s1 = fam[1] * (g[0] + g[2] - r1) + fbm[1] * (rv[0] + g[3] - r1) + fcm[1] * (rv[1] + g[4] - r1)
            s2 = fam[2] * (g[1] + g[3] - r2) + fbm[2] * (g[0] + g[4] - r2) + fcm[2] * (rv[0] + g[5] - r2)
            if side == 0:
                sb[0], sb[1], sb[2] = s0, s1, s2
            else:
                sb[L - 1], sb[L - 2], sb[L - 3] = s0, s1, s2
    else:
        def send(ip):
            sap = [f[L - 1 - (i + 1)] if ip == 1 else f[i + 1] for i in range(LMF + 1)]
            return (sum(pbco[1, 0, i] * sap[i] for i in range(LMF + 1)),
                    sum(pbco[1, 1, i] * sap[i] for i in range(LMF + 1)), sap[0])
        r0, r1 = send(1), send(0)
        sb[0] = sum(pbci[1, 0, q] * f[q] for q in range(LMF + 1)) + r0[0]
        sb[1] = sum(pbci[1, 1, q] * f[q] for q in range(LMF + 1)) + r0[1]
        t = 2 * f[2]
        sb[2] = fa * (f[1] + f[3] - t) + fb * (f[0] + f[4] - t) + fc * (r0[2] + f[5] - t)
        sb[L - 1] = sum(pbci[1, 0, q] * f[L - 1 - q] for q in range(LMF + 1)) + r1[0]
        sb[L - 2] = sum(pbci[1, 1, q] * f[L - 1 - q] for q in range(LMF + 1)) + r1[1]
        t = 2 * f[L - 3]
        sb[L - 3] = fa * (f[L - 4] + f[L - 2] - t) + fb * (f[L - 5] + f[L - 1] - t) + fc * (f[L - 6] + r1[2] - t)
    for i in range(3, L - 3):
        t = 2 * f[i]
        sb[i] = fa * (f[i - 1] + f[i + 1] - t) + fb * (f[i - 2] + f[i + 2] - t) + fc * (f[i - 3] + f[i + 3] - t)
    return sb


def operators(L, periodic, fltk, fltkbc):
    pbci, pbco = sbcco(fltk)
    ns = 1 if periodic else 0
    A = lhs(L, ALBED[ns], ALBED[ns], alpha, beta)
    I = np.eye(L)
    B = np.stack([deriv_rhs(I[:, j], periodic, pbci, pbco) for j in range(L)], axis=1)
    D = np.linalg.solve(A, B)
    frows = filter_rows(fltk, fltkbc)
    al, be, fa, fb, fc = fcint(fltk, 0.5)
    if periodic:
        rs = [[0, 0, 1, al, be], [0, al, 1, al, be], [be, al, 1, al, be]]
    else:
        rs = [r[0] for r in frows]
    Af = lhs(L, rs, rs, al, be)
    Bf = np.stack([filter_rhs(I[:, j], periodic, pbci, pbco, frows, (fa, fb, fc)) for j in range(L)], axis=1)
    G = np.eye(L) + np.linalg.solve(Af, Bf)
    return D, G, pbci, pbco


def main():
    fltk = fltkbc = math.pi * 0.85
    out = {}
    # line lengths of the small test case: xi 25/65 and eta 17 one-sided, zeta 13 periodic
    for L, per in ((25, False), (65, False), (17, False), (13, True), (20, True)):
        D, G, pbci, pbco = operators(L, per, fltk, fltkbc)
        tag = f"{'p' if per else 'o'}{L}"
        out[f"deriv_{tag}"] = D
        out[f"filter_{tag}"] = G
    out["pbci"], out["pbco"] = sbcco(fltk)
    np.savez_compressed(os.path.join(HERE, "line_operators.npz"), **out)
    print("wrote", os.path.join(HERE, "line_operators.npz"), sorted(out))


if __name__ == "__main__":
    main()
