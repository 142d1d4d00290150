"""Six-block H-type aerofoil grid: a numpy restatement of gridaerofoil
(src/Grid.f90:62-482) with its helpers gridf (src/Subroutineso.f90:288-314),
hermite2D (src/Grid.f90:485-583), naca (:696-711), inter/inter2 (:714-755),
drvbn (:758-768), hermite/fillh (:659-693).

Differences from the reference, each a parameter rather than a change of
algorithm: the NACA 00tt thickness is an argument (the reference hard-codes
thk=21, src/Grid.f90:75), and the routine returns the per-block coordinate
arrays instead of writing misc/gridNNN.dat.  Single-precision literals of the
reference (``0.7e0``, the NACA coefficients, ...) are kept single precision,
because Fortran evaluates them in default real.

The grid is host-side set-up: it runs once per case and produces the
``xyz(0:lmx,3)`` planes that ati_set_grid takes.
"""
import math

import numpy as np

from .config import CaseConfig

SML = 1.0e-6
HALF = 0.5
PI = math.pi
PI4 = PI / 4.0


def f32(v):
    """A Fortran default-real literal, promoted to double."""
    return float(np.float32(v))


def gridf(x, xxi, xo, xn, dxo, dxn, mxin, ip):
    """Quintic grid line with end spacings (src/Subroutineso.f90:288-314)."""
    dxoo, dxnn = dxo, dxn
    if dxo == SML:
        dxoo = 2 * (xn - xo) / mxin - dxn
    if dxn == SML:
        dxnn = 2 * (xn - xo) / mxin - dxo
    aa = 6 * (xn - xo) - 3 * mxin * (dxoo + dxnn)
    bb = 15 * (xo - xn) + mxin * (8 * dxoo + 7 * dxnn)
    cc = 10 * (xn - xo) - mxin * (6 * dxoo + 4 * dxnn)
    dd = mxin * dxoo
    fctr = 1.0 / mxin
    for i in range(mxin + 1):
        ii = i + ip
        xi = i * fctr
        x[ii] = aa * xi ** 5 + bb * xi ** 4 + cc * xi ** 3 + dd * xi + xo
        xxi[ii] = fctr * (5 * aa * xi ** 4 + 4 * bb * xi ** 3 + 3 * cc * xi ** 2 + dd)


def naca(x, c, t0, n):
    """NACA 00xx half-thickness (src/Grid.f90:696-711)."""
    t = t0 * f32(0.01)
    k = f32(0.991148635)
    xc = x / c
    y = (t * c * k / f32(0.2)) * (f32(0.298222773) * math.sqrt(xc) - f32(0.127125232) * xc
                                  - f32(0.357907906) * xc ** 2 + f32(0.291984971) * xc ** 3
                                  - f32(0.105174606) * xc ** 4)
    if n == 0:
        y = -1.0 * y
    return y


def inter(k01, k02, k03, k04, x0, x1, x):
    l = x1 - x0
    invl = 1.0 / l
    fx = (x - x0) * invl
    a = (2 * fx ** 3 - 3 * fx ** 2 + 0 * fx + 1)
    b = (1 * fx ** 3 - 2 * fx ** 2 + 1 * fx + 0)
    c = (-2 * fx ** 3 + 3 * fx ** 2 + 0 * fx + 0)
    d = (1 * fx ** 3 - 1 * fx ** 2 + 0 * fx + 0)
    return a * k01 + b * l * k02 + c * k03 + d * l * k04


def inter2(k01, k02, k03, k04, x0, x1, x, side):
    l = x1 - x0
    invl = 1.0 / l
    fx = (x - x0) * invl
    if side == 1:
        a = (-3 * fx ** 4 + 8 * fx ** 3 - 6 * fx ** 2 + 0 * fx + 1)
        b = (-1 * fx ** 4 + 3 * fx ** 3 - 3 * fx ** 2 + 1 * fx + 0)
        d = (-2 * fx ** 4 + 5 * fx ** 3 - 3 * fx ** 2 + 0 * fx + 0)
        c = (3 * fx ** 4 - 8 * fx ** 3 + 6 * fx ** 2 + 0 * fx + 0)
    else:
        a = (3 * fx ** 4 - 4 * fx ** 3 + 0 * fx ** 2 + 0 * fx + 1)
        b = (2 * fx ** 4 - 3 * fx ** 3 + 0 * fx ** 2 + 1 * fx + 0)
        d = (1 * fx ** 4 - 1 * fx ** 3 + 0 * fx ** 2 + 0 * fx + 0)
        c = (-3 * fx ** 4 + 4 * fx ** 3 + 0 * fx ** 2 + 0 * fx + 0)
    return a * k01 + b * l * k02 + c * k03 + d * l * k04


def fillh(u):
    a0 = 2 * u ** 3 - 3 * u ** 2 + 0 * u + 1
    a1 = -2 * u ** 3 + 3 * u ** 2 + 0 * u + 0
    b0 = 1 * u ** 3 - 2 * u ** 2 + 1 * u + 0
    b1 = 1 * u ** 3 - 1 * u ** 2 + 0 * u + 0
    return a0, a1, b0, b1


def hermite(k01, k02, k03, k04, lx, x):
    l = float(lx)
    invl = 1.0 / l
    v = fillh(x * invl)
    return v[0] * k01 + v[2] * l * k02 + v[1] * k03 + v[3] * l * k04


def drvbn(x, side):
    if side == 0:
        return (-1.5) * x[0] + 2.0 * x[1] - 0.5 * x[2]
    return 1.5 * x[-1] - 2.0 * x[-2] + 0.5 * x[-3]


def hermite2d(xx, yy, is_, ie, js, je):
    """Coons patch with Hermite blending, updated in place row by row as the
    reference does (src/Grid.f90:485-583)."""
    lxi, let = ie - is_, je - js
    xv = np.zeros((lxi + 1, 2)); yv = np.zeros((lxi + 1, 2))
    xu = np.zeros((let + 1, 2)); yu = np.zeros((let + 1, 2))
    for side in (0, 1):
        xv[0, side] = drvbn(xx[is_, js:je + 1], side)
        xv[lxi, side] = drvbn(xx[ie, js:je + 1], side)
        yv[0, side] = drvbn(yy[is_, js:je + 1], side)
        yv[lxi, side] = drvbn(yy[ie, js:je + 1], side)
        xu[0, side] = drvbn(xx[is_:ie + 1, js], side)
        xu[let, side] = drvbn(xx[is_:ie + 1, je], side)
        yu[0, side] = drvbn(yy[is_:ie + 1, js], side)
        yu[let, side] = drvbn(yy[is_:ie + 1, je], side)
    for i in range(lxi + 1):
        for arr in (xv, yv):
            arr[i, 0] = hermite(arr[0, 0], 0.0, arr[lxi, 0], 0.0, lxi, i)
            arr[i, 1] = hermite(arr[0, 1], 0.0, arr[lxi, 1], 0.0, lxi, i)
    for i in range(let + 1):
        for arr in (xu, yu):
            arr[i, 0] = hermite(arr[0, 0], 0.0, arr[let, 0], 0.0, let, i)
            arr[i, 1] = hermite(arr[0, 1], 0.0, arr[let, 1], 0.0, let, i)
    mx = np.array([[xx[is_, js], xx[is_, je], xv[0, 0], xv[0, 1]],
                   [xx[ie, js], xx[ie, je], xv[lxi, 0], xv[lxi, 1]],
                   [xu[0, 0], xu[let, 0], 0.0, 0.0],
                   [xu[0, 1], xu[let, 1], 0.0, 0.0]])
    my = np.array([[yy[is_, js], yy[is_, je], yv[0, 0], yv[0, 1]],
                   [yy[ie, js], yy[ie, je], yv[lxi, 0], yv[lxi, 1]],
                   [yu[0, 0], yu[let, 0], 0.0, 0.0],
                   [yu[0, 1], yu[let, 1], 0.0, 0.0]])
    uu = np.arange(lxi + 1, dtype=np.float64) / lxi
    hu = np.stack(fillh(uu))          # (4, lxi+1)
    for j in range(js, je + 1):
        jj = j - js
        hv = fillh(float(jj) / let)
        for xy, m, vd in ((xx, mx, xu), (yy, my, yu)):
            v = (xy[is_, j], xy[ie, j], vd[jj, 0], vd[jj, 1])
            ux = (xy[is_:ie + 1, js].copy(), xy[is_:ie + 1, je].copy(),
                  (xv if xy is xx else yv)[:, 0], (xv if xy is xx else yv)[:, 1])
            val1 = hu[0] * v[0] + hu[1] * v[1] + hu[2] * v[2] + hu[3] * v[3]
            val2 = ux[0] * hv[0] + ux[1] * hv[1] + ux[2] * hv[2] + ux[3] * hv[3]
            mh = [m[r, 0] * hv[0] + m[r, 1] * hv[1] + m[r, 2] * hv[2] + m[r, 3] * hv[3] for r in range(4)]
            val3 = hu[0] * mh[0] + hu[1] * mh[1] + hu[2] * mh[2] + hu[3] * mh[3]
            xy[is_:ie + 1, j] = val1 + val2 - val3


def aerofoil_grid(cfg: CaseConfig):
    """Per-block coordinates [x, y, z] for a bkx=3, bky=2, bkz=1 H-grid.

    Returns a list over blocks mb = j*bkx + i of float64 arrays shaped
    (3, lze+1, let+1, lxi+1): C order equals the Fortran xyz(0:lmx,3)."""
    lxibk, letbk, lzebk = list(cfg.lxibk), list(cfg.letbk), list(cfg.lzebk)
    bkx, bky = len(lxibk), len(letbk)
    if bkx != 3 or bky != 2 or len(lzebk) != 1:
        raise ValueError("the aerofoil H-grid has 3x2x1 blocks")
    nthick = 2
    smgrid, domlen, span = cfg.smgrid, cfg.domlen, cfg.span
    wlew, wlea, szth1, szth2, szxt = cfg.wlew, cfg.wlea, cfg.szth1, cfg.szth2, cfg.szxt
    c1, delt1 = cfg.chord, math.radians(cfg.delt_deg)
    thk = cfg.thick
    lxit = sum(lxibk) + (bkx - 1)
    lett = sum(letbk) + (bky - 1)
    lxise = [[0, lxibk[0]]]
    for i in range(1, bkx):
        s = lxise[i - 1][1] + 1
        lxise.append([s, s + lxibk[i]])
    letse = [[0, letbk[0]]]
    for j in range(1, bky):
        s = letse[j - 1][1] + 1
        letse.append([s, s + letbk[j]])
    lze = lzebk[0]
    shs1 = cfg.ximod * smgrid
    shs2 = cfg.etamod * smgrid
    she1 = shs2
    smod = (4, 3)
    npy = min(nthick, 1) + bky
    npx = bkx
    xx = np.zeros((lxit + 1, lett + 1)); yy = np.zeros((lxit + 1, lett + 1))
    xp = np.zeros((lxit + 1, npy + 1)); yp = np.zeros((lxit + 1, npy + 1))
    xq = np.zeros((lett + 1, npx + 1)); yq = np.zeros((lett + 1, npx + 1))
    pxi = np.zeros((lxit + 1, npy + 1)); qet = np.zeros((lett + 1, npx + 1))
    px = np.zeros((bkx + 3, npy + 1)); py = np.zeros((npy + 3, npx + 1))
    hslo = np.zeros((npy + 1, bkx, 2)); vslo = np.zeros((npx + 1, bky, 2))
    dlth = [[f32(0.7) * domlen, domlen + szxt], [f32(0.7) * domlen, domlen + szxt]]
    szth = [[szth1, szth2 + szxt], [szth1, szth2 + szxt]]
    degarr = [None, 25 * PI / 180, 0 * PI / 180, 15 * PI / 180]
    nwk = [int(np.float32(lxibk[2]) * np.float32(0.45)), int(np.float32(letbk[1]) * np.float32(0.4))]
    nwk2 = [int(np.float32(0.9) * np.float32(nwk[0])), int(np.float32(1.0) * np.float32(nwk[1]))]
    lwk = [f32(1.5) * c1, f32(0.5) * c1]
    lwk2 = [1.5 * lwk[0], f32(1.8) * lwk[1]]
    lhbl = [0.15 * c1, 0.15 * c1]
    lvbl = [HALF * lwk[1], lwk[1]]
    nvbl = [int(np.float32(letbk[0]) * np.float32(0.3)), nwk[1]]
    zs = np.array([span * (float(lze - k) / lze - HALF) for k in range(lze + 1)])
    blocks = []
    for mb in range(bkx * bky):
        a, b = lxibk[mb % bkx], letbk[mb // bkx]
        blocks.append(np.zeros((3, lze + 1, b + 1, a + 1)))
    plane_cache = None
    for k in range(lze + 1):
        lwle = wlea * math.sin(2 * PI * (zs[k] - zs[0]) / wlew)
        if plane_cache is not None and wlea == 0.0:
            xx, yy = plane_cache
        else:
            px[0, :] = -dlth[0][0]
            px[1, :] = px[0, :] + szth[0][0]
            px[2, 1:3] = -HALF * c1 + lwle * math.cos(delt1)
            px[2, 0] = px[2, 2] - lhbl[0]
            px[2, 3] = px[2, 2] - lhbl[1]
            px[3, :] = -HALF * c1 + c1 * math.cos(delt1)
            px[3, 3] = px[3, 2]
            px[4, :] = px[3, 0] + dlth[0][1] - szth[0][1]
            px[5, :] = px[3, 0] + dlth[0][1]
            py[0, :] = -dlth[1][0]
            py[1, :] = py[0, :] + szth[1][0]
            py[2, 0] = 0.0
            py[2, 1] = -lwle * math.sin(delt1)
            py[2, 2] = -c1 * math.sin(delt1)
            py[2, 3] = py[2, 2]
            py[3, :] = py[2, :]
            py[4, :] = py[2, 2] + dlth[1][1] - szth[1][1]
            py[5, :] = py[2, 2] + dlth[1][1]
            hslo[:] = 0.0
            hslo[1, 0, :] = (0.0, -math.tan(delt1))
            hslo[1, 2, :] = (-math.tan(delt1 + 2 * degarr[2]), 0.0)
            vslo[:] = 0.0
            vslo[1, 0, :] = (0.0, math.tan(PI4 + delt1))
            vslo[1, 1, :] = (-math.tan(PI4 - delt1), 0.0)
            ra1 = 0.0
            # horizontal lines: x (src/Grid.f90:213-272)
            for n in range(npy + 1):
                ip, im = lxise[0][0], lxibk[0]
                if n == 0 or n == npy:
                    gridf(xp[:, n], pxi[:, n], px[0, n], px[2, n], 220 * shs1, shs1 * smod[0], im, ip)
                else:
                    gridf(xp[:, n], pxi[:, n], px[0, n], px[2, n], 220 * shs1, shs1, im, ip)
                if n in (0, 3):
                    ip, im = lxise[1][0], lxibk[1]
                    gridf(xp[:, n], pxi[:, n], px[2, n], px[3, n], shs1 * smod[0], she1 * smod[0], im, ip)
                if n != npy:
                    ip, im = lxise[2][0], nwk[0]
                    tmpa, sha, tmpb, shb = px[3, n], she1, px[3, n] + lwk[0], SML
                    ra0 = sha
                    gridf(xp[:, n], pxi[:, n], tmpa, tmpb, sha, shb, im, ip)
                    ip = ip + im
                    im = lxibk[2] - im
                    tmpa, sha, tmpb, shb = tmpb, pxi[ip, n], px[5, n], 200 * ra0
                    gridf(xp[:, n], pxi[:, n], tmpa, tmpb, sha, shb, im, ip)
                    if n == npy - 1:
                        ra1 = shb
                else:
                    ip, im = lxise[2][0], nwk2[0]
                    tmpa, sha = px[3, n], she1 * smod[0]
                    ra0 = sha
                    tmpb, shb = px[3, n] + lwk2[0], SML
                    gridf(xp[:, n], pxi[:, n], tmpa, tmpb, sha, shb, im, ip)
                    ip = ip + im
                    im = lxibk[2] - im
                    tmpa, sha, tmpb, shb = tmpb, pxi[ip, n], px[5, n], f32(1.2) * ra1
                    gridf(xp[:, n], pxi[:, n], tmpa, tmpb, sha, shb, im, ip)
            # horizontal lines: y (src/Grid.f90:276-297)
            yp[:, 0] = py[0, 0]
            k01, k03, k02, k04 = py[2, 0], py[2, 1], hslo[1, 0, 0], hslo[1, 0, 1]
            x0, x1 = px[0, 1], px[2, 1]
            for i in range(lxise[0][0], lxise[0][1] + 1):
                yp[i, 1] = inter(k01, k02, k03, k04, x0, x1, xp[i, 1])
                yp[i, 2] = yp[i, 1]
            k01, k03, k02, k04 = py[2, 2], py[2, 3], hslo[1, 2, 0], hslo[1, 2, 1]
            x0, x1 = px[3, 1], px[5, 1]
            for i in range(lxise[2][0], lxise[2][1] + 1):
                yp[i, 1] = inter2(k01, k02, k03, k04, x0, x1, xp[i, 1], 1)
                yp[i, 2] = yp[i, 1]
            yp[:, 3] = py[5, 0]
            # aerofoil surface (src/Grid.f90:300-330)
            tmp, tmpa, tmpb = c1 - lwle, px[2, 1], py[2, 1]
            lxis, lxie, lxib = lxise[1][0], lxise[1][1], lxibk[1]
            alph = delt1
            for n in (1, 2):
                yp[lxis, n] = 0.0
                xp[lxis, n] = 0.0
                ll = 25
                for i in range(lxis + 1, lxis + ll + 1):
                    xp[i, n] = xp[i - 1, n] + HALF * shs1
                    err = 1.0
                    while abs(err) > SML:
                        yp[i, n] = naca(xp[i, n], tmp, thk, n - 1)
                        err = math.sqrt((xp[i, n] - xp[i - 1, n]) ** 2 + (yp[i, n] - yp[i - 1, n]) ** 2) / shs1 - 1
                        xp[i, n] = xp[i, n] - HALF ** 8 * err * shs1
                xo = xp[lxis + ll, n]
                w = (3, -16, 36, -48, 25)
                sho = sum(xp[lxis + ll - 4 + q, n] * w[q] for q in range(5)) / 12
                ip, im = lxis + ll, lxib - ll
                gridf(xp[:, n], pxi[:, n], xo, tmp, sho, she1, im, ip)
                for i in range(lxis + ll + 1, lxie):
                    yp[i, n] = naca(xp[i, n], tmp, thk, n - 1)
                yp[lxie, n] = 0.0
                for i in range(lxis, lxie + 1):
                    oxp, oyp = xp[i, n], yp[i, n]
                    xp[i, n] = (oxp * math.cos(alph) + oyp * math.sin(alph)) + tmpa
                    yp[i, n] = (-oxp * math.sin(alph) + oyp * math.cos(alph)) + tmpb
            # vertical lines: y (src/Grid.f90:334-382)
            ra2 = 0.0
            for n in range(bkx + 1):
                if n != bkx:
                    im = nvbl[0]
                    ip = letse[0][1] - im
                    gridf(yq[:, n], qet[:, n], py[2, n] - lvbl[0], py[2, n], SML,
                          shs2 * math.cos(PI4 + delt1), im, ip)
                    ip = letse[0][0]
                    im = letbk[0] - im
                    gridf(yq[:, n], qet[:, n], py[0, n], py[2, n] - lvbl[0], SML, qet[im, n], im, ip)
                    if n == bkx - 1:
                        ra2 = qet[letse[0][0], n]
                    ip, im = letse[1][0], nwk[1]
                    tmpa, sha, tmpb, shb = py[2, n], shs2 * math.cos(PI4 - delt1), py[2, n] + lvbl[1], SML
                    gridf(yq[:, n], qet[:, n], tmpa, tmpb, sha, shb, im, ip)
                    ip = ip + im
                    im = letbk[1] - im
                    tmpa, sha, tmpb, shb = tmpb, qet[ip, n], py[5, n], SML
                    gridf(yq[:, n], qet[:, n], tmpa, tmpb, sha, shb, im, ip)
                    if n == bkx - 1:
                        ra1 = qet[letse[1][1], n]
                else:
                    im = int(HALF * nwk2[1])
                    ip = letse[0][1] - im
                    gridf(yq[:, n], qet[:, n], py[2, n] - lwk2[1], py[2, n], SML,
                          shs2 * math.cos(PI4 + delt1) * smod[1], im, ip)
                    ip = letse[0][0]
                    im = letbk[0] - im
                    gridf(yq[:, n], qet[:, n], py[0, n], py[2, n] - lwk2[1], ra2 * f32(0.9), qet[im, n], im, ip)
                    ip, im = letse[1][0], nwk2[1]
                    tmpa, sha = py[2, n], shs2 * math.cos(PI4 - delt1) * smod[1]
                    tmpb, shb = py[2, n] + lwk2[1], SML
                    gridf(yq[:, n], qet[:, n], tmpa, tmpb, sha, shb, im, ip)
                    ip = ip + im
                    im = lett - ip
                    tmpa, sha, tmpb, shb = tmpb, qet[ip, n], py[5, n], ra1 * f32(1.2)
                    gridf(yq[:, n], qet[:, n], tmpa, tmpb, sha, shb, im, ip)
            # vertical lines: x (src/Grid.f90:386-430)
            xq[:, 0] = px[0, 0]
            xq[letse[0][0]:letse[0][1] + 1, 1] = px[2, 0]
            is_, ie = letbk[0] - nvbl[0], letse[0][1]
            k01, k03, k02, k04 = px[2, 0], px[2, 1], vslo[1, 0, 0], vslo[1, 0, 1]
            x0, x1 = yq[is_, 1], yq[ie, 1]
            for i in range(is_, ie + 1):
                xq[i, 1] = inter2(k01, k02, k03, k04, x0, x1, yq[i, 1], 0)
            xq[letse[1][0]:letse[1][1] + 1, 1] = px[2, 3]
            is_, ie = letse[1][0], letse[1][0] + nvbl[1]
            k01, k03, k02, k04 = px[2, 2], px[2, 3], vslo[1, 1, 0], vslo[1, 1, 1]
            x0, x1 = yq[is_, 1], yq[ie, 1]
            for i in range(is_, ie + 1):
                xq[i, 1] = inter2(k01, k02, k03, k04, x0, x1, yq[i, 1], 1)
            is_, ie = letse[0][0], letse[0][1]
            k01, k03, k02, k04 = px[3, 0], px[3, 1], vslo[2, 0, 0], vslo[2, 0, 1]
            x0, x1 = yq[is_, 2], yq[ie, 2]
            for i in range(is_, ie + 1):
                xq[i, 2] = inter2(k01, k02, k03, k04, x0, x1, yq[i, 2], 0)
            is_, ie = letse[1][0], letse[1][1]
            k01, k03, k02, k04 = px[3, 2], px[3, 3], vslo[2, 1, 0], vslo[2, 1, 1]
            x0, x1 = yq[is_, 2], yq[ie, 2]
            for i in range(is_, ie + 1):
                xq[i, 2] = inter2(k01, k02, k03, k04, x0, x1, yq[i, 2], 1)
            xq[:, 3] = px[5, 0]
            # block patches (src/Grid.f90:434-448)
            xx = np.zeros((lxit + 1, lett + 1)); yy = np.zeros((lxit + 1, lett + 1))
            linesy = (0, 2)
            for l in range(bky):
                js, je = letse[l]
                n = linesy[l]
                for m in range(bkx):
                    is_, ie = lxise[m]
                    xx[is_:ie + 1, js] = xp[is_:ie + 1, n]; xx[is_:ie + 1, je] = xp[is_:ie + 1, n + 1]
                    yy[is_:ie + 1, js] = yp[is_:ie + 1, n]; yy[is_:ie + 1, je] = yp[is_:ie + 1, n + 1]
                    xx[is_, js:je + 1] = xq[js:je + 1, m]; xx[ie, js:je + 1] = xq[js:je + 1, m + 1]
                    yy[is_, js:je + 1] = yq[js:je + 1, m]; yy[ie, js:je + 1] = yq[js:je + 1, m + 1]
                    hermite2d(xx, yy, is_, ie, js, je)
            plane_cache = (xx, yy)
        for mb in range(bkx * bky):
            js, je = letse[mb // bkx]
            is_, ie = lxise[mb % bkx]
            blocks[mb][0, k] = xx[is_:ie + 1, js:je + 1].T
            blocks[mb][1, k] = yy[is_:ie + 1, js:je + 1].T
            blocks[mb][2, k] = zs[k]
    return blocks


def min_cell_jacobian(blocks):
    """Sign check used by tests and bench: the 2-D cell areas of every block
    plane must keep one sign (no folded cells)."""
    out = []
    for xyz in blocks:
        x, y = xyz[0, 0], xyz[1, 0]
        a = (x[1:, 1:] - x[:-1, :-1]) * (y[:-1, 1:] - y[1:, :-1]) - (y[1:, 1:] - y[:-1, :-1]) * (x[:-1, 1:] - x[1:, :-1])
        out.append((float(a.min()), float(a.max())))
    return out
