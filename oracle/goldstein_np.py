"""ORACLE -- test infrastructure only (never imported by the product).

Second, independent restatement of the reference GOLDSTEIN tracer step in
NumPy, written separately from oracle/goldstein_oracle.c and structured
differently: the flux step of src/goldstein/goldstein.f90:2436-2642 is
vectorised over a whole level (the sequential carries fw/fs/fb of the
reference become shifted face arrays), and the convective adjustment of
goldstein.f90:2657-2841 is a per-column Python routine.  Each element-wise
expression keeps the reference's operation order, so results are expected to
be bit-identical to the C restatement; the tests check that.

Arrays use the C-order views described in cgenie_gb300/grid.py
(``ts[k, j, i, l]`` is Fortran ``ts(l, i, j, k)``).
"""
from __future__ import annotations

import numpy as np


def eos(ec, t, s, z, ieos):
    """goldstein.f90:3048-3061"""
    if ieos == 0:
        return ec[0] * t + ec[1] * s + ec[2] * (t * t) + ec[3] * ((t * t) * t)
    return ec[0] * t + ec[1] * s + ec[2] * (t * t) + ec[3] * ((t * t) * t) + ec[4] * t * z


def eosd(ec, t1, t2, s1, s2, z, rdz, ieos):
    """goldstein.f90:3064-3082 -> (dzrho, tec)"""
    tatw = 0.5 * (t1 + t2)
    if ieos == 0:
        tec = -ec[0] - ec[2] * tatw * 2 - ec[3] * tatw * tatw * 3
    else:
        tec = -ec[0] - ec[2] * tatw * 2 - ec[3] * tatw * tatw * 3 - ec[4] * z
    dzrho = (ec[1] * (s2 - s1) - tec * (t2 - t1)) * rdz
    return dzrho, tec


class Params:
    def __init__(self, m, diso, ieos, iconv, iediff, imld=0):
        self.diff = m.diff
        self.ec = m.ec
        self.diso = bool(diso)
        self.ieos = ieos
        self.iconv = iconv
        self.iediff = iediff
        self.ediff0 = m.ediff0
        self.ediffpow2 = m.ediffpow2
        self.ediffpow2i = m.ediffpow2i
        self.imld = imld
        self.mldpebuoycoeff = getattr(m.cfg, "mldpebuoycoeff", 0.15)


def flux(m, p, ts, ts1, rho, u):
    """tstepo_flux (goldstein.f90:2436-2642), vectorised per level.  Updates ts
    (wet interior) and rho (all interior) in place; returns (dmax, limps)."""
    maxi, maxj, maxk, L = m.maxi, m.maxj, m.maxk, m.maxl
    ec = p.ec
    d1, d2 = p.diff[0], p.diff[1]
    J = slice(1, maxj + 1)
    I = slice(1, maxi + 1)
    k1 = m.k1
    k1c = k1[J, I]                                   # (maxj, maxi)
    # i+1 neighbour with the reference's doorway: column 1 for i = maxi
    ip = np.arange(2, maxi + 2)
    ip[-1] = 1
    k1e = k1[J][:, ip]
    k1n = k1[2:maxj + 2, I]
    rc = m.rc[1:maxj + 1][:, None]
    rc2 = m.rc2[1:maxj + 1][:, None]
    cvj = m.cv[1:maxj + 1][:, None]
    cv2p = np.zeros(maxj + 1)
    cv2p[1:maxj] = m.cv2[: maxj - 1]
    cv2j = cv2p[1:maxj + 1][:, None]
    dsvp = np.zeros(maxj + 1)
    dsvp[1:maxj] = m.dsv[: maxj - 1]
    dsv_min = np.array([dsvp[min(j, maxj - 1)] for j in range(1, maxj + 1)])[:, None]
    rdsvp = np.zeros(maxj + 1)                       # rdsv(0:maxj), ends unused (masked)
    rdsvp[1:maxj] = m.rdsv[: maxj - 1]
    rdsj = m.rds[:maxj][:, None]
    dmax = 0.0
    limps = 0
    fa_prev = np.zeros((maxj, maxi, L))
    scc = ec[1] if p.diso else 0.0
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        for k in range(1, maxk + 1):
            T1 = ts1[k]                               # (NJ, NI, L)
            Tc = T1[J, I]
            uk = u[k - 1]
            u1 = uk[J, I, 0][:, :, None]
            u2 = uk[J, I, 1][:, :, None]
            u3 = uk[J, I, 2][:, :, None]
            dza = m.dza[k - 1]
            rdza = m.rdza[k - 1]
            # per-cell vertical density gradient and diffusivity
            wet_v = (k >= k1c) & (k < maxk)
            if k < maxk:
                dzrho, tec = eosd(ec, Tc[:, :, 0], ts1[k + 1][J, I, 0], Tc[:, :, 1], ts1[k + 1][J, I, 1],
                                  m.zw[k], rdza, p.ieos)
            else:
                dzrho = np.zeros((maxj, maxi))
                tec = np.zeros((maxj, maxi))
            rdzrho = np.where(dzrho < -1.0e-12, 1.0 / dzrho, -1.0e12)
            diffv = np.full((maxj, maxi), d2)
            if p.iediff in (1, 2) and k < maxk:
                e1 = m.ediff1[k - 1]
                if p.ediffpow2i == 0:
                    dv = p.ediff0 + e1
                elif p.ediffpow2i == 1:
                    dv = p.ediff0 + e1 * (-rdzrho)
                elif p.ediffpow2i == 2:
                    dv = p.ediff0 + e1 * np.sqrt(-rdzrho)
                else:
                    dv = p.ediff0 + e1 * np.power(-rdzrho, p.ediffpow2)
                dv = np.where(dv > m.diffmax[k], m.diffmax[k], dv)
                diffv = np.where(wet_v, dv, diffv)
            pec1 = u1 * m.dphi / d1
            ups1 = pec1 / (2.0 + np.abs(pec1))
            pec2 = u2 * dsv_min[:, :, None] / d1
            ups2 = pec2 / (2.0 + np.abs(pec2))
            pec3 = u3 * dza / diffv[:, :, None]
            ups3 = pec3 / (2.0 + np.abs(pec3))
            # east faces (the i = maxi face is the western doorway of i = 1)
            Te = T1[J][:, ip, :]
            fe = u1 * rc[:, :, None] * ((1.0 - ups1) * Te + (1.0 + ups1) * Tc) * 0.5
            fe = fe - (Te - Tc) * rc2[:, :, None] * d1
            fe = np.where((k >= np.maximum(k1c, k1e))[:, :, None], fe, 0.0)
            fw = np.concatenate([fe[:, -1:, :], fe[:, :-1, :]], axis=1)
            # north faces
            Tn = T1[2:maxj + 2, I]
            fn = cvj[:, :, None] * u2 * ((1.0 - ups2) * Tn + (1.0 + ups2) * Tc) * 0.5
            fn = fn - cv2j[:, :, None] * (Tn - Tc) * d1
            fn = np.where((k >= np.maximum(k1c, k1n))[:, :, None], fn, 0.0)
            fs = np.concatenate([np.zeros((1, maxi, L)), fn[:-1]], axis=0)
            # faces above
            if k == maxk:
                fa = np.broadcast_to(ts[maxk + 1][J, I], (maxj, maxi, L)).copy()
            else:
                Ta = ts1[k + 1][J, I]
                fa = u3 * ((1.0 - ups3) * Ta + (1.0 + ups3) * Tc) * 0.5
                fa = fa - (Ta - Tc) * rdza * diffv[:, :, None]
            fa = np.where((k >= k1c)[:, :, None], fa, 0.0)
            if p.diso and k < maxk:
                act = wet_v & (dzrho < -1.0e-12)
                tv1 = np.zeros((maxj, maxi))
                dxts = []
                dyts = []
                dxr = []
                dyr = []
                for knp in (0, 1):
                    Tk = ts1[k + knp]
                    for nnp in (0, 1):
                        mx = (k + knp >= k1[J, nnp * 2:maxi + nnp * 2])     # k1(i-1+2nnp, j)
                        dx = (Tk[J, 1 + nnp:maxi + 1 + nnp] - Tk[J, nnp:maxi + nnp]) * rc[:, :, None] * m.rdphi
                        dx = np.where(mx[:, :, None], dx, 0.0)
                        my = (k + knp >= k1[nnp * 2:maxj + nnp * 2, I])     # k1(i, j-1+2nnp)
                        cvv = m.cv[nnp:maxj + nnp][:, None, None]           # cv(j-1+nnp)
                        rsv = rdsvp[nnp:maxj + nnp][:, None, None]          # rdsv(j+nnp-1)
                        dy = (Tk[1 + nnp:maxj + 1 + nnp, I] - Tk[nnp:maxj + nnp, I]) * cvv * rsv
                        dy = np.where(my[:, :, None], dy, 0.0)
                        xr = scc * dx[:, :, 1] - tec * dx[:, :, 0]
                        yr = scc * dy[:, :, 1] - tec * dy[:, :, 0]
                        tv1 = tv1 + xr * xr + yr * yr
                        dxts.append(dx)
                        dyts.append(dy)
                        dxr.append(xr)
                        dyr.append(yr)
                tv1 = 0.25 * tv1 * rdzrho * rdzrho
                ss = m.ssmax[k - 1]
                lim = tv1 > ss
                slim = np.where(lim, ss * ss / (tv1 * tv1), 1.0)
                limps += int(np.count_nonzero(lim & act))
                tv1b = tv1 * slim * d1 * rdza
                tvd = tv1b * m.dt[k - 1] * rdza
                if np.any(act):
                    dmax = max(dmax, float(np.max(np.where(act, tvd, 0.0))))
                dzts = (ts1[k + 1][J, I] - Tc) * rdza
                tv = np.zeros((maxj, maxi, L))
                dz2 = (2 * dzrho)[:, :, None]
                for n in range(4):
                    xr = dxr[n][:, :, None]
                    yr = dyr[n][:, :, None]
                    tv = tv + (dz2 * dxts[n] - xr * dzts) * xr + (dz2 * dyts[n] - yr * dzts) * yr
                tv = 0.25 * slim[:, :, None] * d1 * tv / (dzrho * dzrho)[:, :, None]
                fa = np.where(act[:, :, None], fa + tv, fa)
            new = Tc - m.dt[k - 1] * (-0.0 + (fe - fw) * m.rdphi + (fn - fs) * rdsj[:, :, None]
                                      + (fa - fa_prev) * m.rdz[k - 1])
            ts[k, J, I] = np.where((k >= k1c)[:, :, None], new, ts[k, J, I])
            rho[k, J, I] = eos(ec, ts[k, J, I, 0], ts[k, J, I, 1], m.zro[k - 1], p.ieos)
            fa_prev = fa
    return dmax, limps


def _coshuffle_col(m, p, tv, r, k1):
    """coshuffle for one column; tv[k, l], r[k] (k = 0..maxk+1 / 0..maxk)."""
    maxk = m.maxk
    ec = p.ec
    zw, dz, rdz = m.zw, m.dz, m.rdz
    icos = 0
    k0 = 0
    ipass = 0
    while k0 < maxk and ipass < maxk:
        ipass += 1
        k = maxk - 1
        if p.ieos:
            r[maxk] = eos(ec, tv[maxk, 0], tv[maxk, 1], zw[k], p.ieos)
            r[k] = eos(ec, tv[k, 0], tv[k, 1], zw[k], p.ieos)
        while r[maxk] > r[k] and k >= k1:
            k -= 1
            if p.ieos:
                r[maxk] = eos(ec, tv[maxk, 0], tv[maxk, 1], zw[k], p.ieos)
                r[k] = eos(ec, tv[k, 0], tv[k, 1], zw[k], p.ieos)
        k0 = k + 1
        if k0 < maxk:
            top = tv[maxk].copy()
            for kk in range(maxk, k0, -1):
                tv[kk] = ((dz[kk - 1] - dz[maxk - 1]) * tv[kk] + dz[maxk - 1] * tv[kk - 1]) * rdz[kk - 1]
            tv[k0] = ((dz[k0 - 1] - dz[maxk - 1]) * tv[k0] + dz[maxk - 1] * top) * rdz[k0 - 1]
            for kk in range(k0, maxk + 1):
                r[kk] = eos(ec, tv[kk, 0], tv[kk, 1], zw[maxk - 1], p.ieos)
            icos = max(icos, maxk - k0)
    return icos


def _co_col(m, p, tv, r, k1):
    """co main loop + fill for one wet column; returns the number of filled levels."""
    maxk = m.maxk
    ec = p.ec
    zw = m.zw
    idx = [0] * (maxk + 1)       # the reference's k(0:maxk)
    dzm = [0.0] * (maxk + 1)
    idx[k1 - 1] = 0
    for mm in range(k1, maxk + 1):
        idx[mm] = mm
        dzm[mm] = m.dz[mm - 1]

    def refresh(a, b):
        if p.ieos:
            r[idx[a]] = eos(ec, tv[idx[a], 0], tv[idx[a], 1], zw[idx[b]], p.ieos)
            r[idx[b]] = eos(ec, tv[idx[b], 0], tv[idx[b], 1], zw[idx[b]], p.ieos)

    mm = maxk
    lastmix = 0
    while idx[mm - 1] > 0 or (lastmix != 0 and idx[mm] != maxk):
        refresh(mm, mm - 1)
        if r[idx[mm]] < r[idx[mm - 1]] or idx[mm - 1] == 0:
            mm = mm - 1 if (lastmix == 0 or idx[mm] == maxk) else mm + 1
            lastmix = 0
            continue
        lastmix = 1
        n = mm - 1
        refresh(n, n - 1)
        while idx[n - 1] > 0 and r[idx[n]] >= r[idx[n - 1]]:
            n -= 1
            refresh(n, n - 1)
        top = idx[mm]
        acc = tv[top] * dzm[top]
        for ni in range(1, mm - n + 1):
            lev = idx[mm - ni]
            acc = acc + tv[lev] * dzm[lev]
            dzm[top] = dzm[top] + dzm[lev]
        tv[top] = acc / dzm[top]
        r[top] = eos(ec, tv[top, 0], tv[top, 1], zw[idx[mm - 1]], p.ieos)
        shift = mm - n
        ni = mm - 1
        while idx[ni + 1] > 0:
            idx[ni] = idx[ni - shift]
            ni -= 1
    filled = 0
    mm = maxk - 1
    for n in range(maxk - 1, k1 - 1, -1):
        if n > idx[mm]:
            tv[n] = tv[idx[mm + 1]]
            r[n] = eos(ec, tv[n, 0], tv[n, 1], zw[idx[n - 1]], p.ieos)
            filled += 1
        else:
            mm -= 1
    return filled


def co(m, p, ts, rho, cost, icosd):
    """co (goldstein.f90:2657-2777) with coshuffle (goldstein.f90:2781-2841) when iconv == 1."""
    maxi, maxj, maxk = m.maxi, m.maxj, m.maxk
    for j in range(1, maxj + 1):
        for i in range(1, maxi + 1):
            k1 = int(m.k1[j, i])
            if k1 > maxk:
                continue
            tv = ts[:, j, i, :]          # view (maxk+2, L)
            r = rho[:, j, i]             # view (maxk+1,)
            if p.iconv == 1:
                icosd[j - 1, i - 1] = _coshuffle_col(m, p, tv, r, k1)
            filled = _co_col(m, p, tv, r, k1)
            if p.iconv == 1:
                icosd[j - 1, i - 1] = max(icosd[j - 1, i - 1], filled)
                cost[j - 1, i - 1] = 5.0e3 * m.zw[maxk - 1 - icosd[j - 1, i - 1]]
            else:
                cost[j - 1, i - 1] += float(filled)



def _level_pair_grids(zw):
    """goldstein.f90:1013-1025 as functions of (k, kk): dzg = zw(k) - zw(kk-1),
    z2dzg = -zw(k)^2 + zw(kk-1)^2, rdzg = 1/dzg (1e10 where k = kk-1)."""
    def dzg(k, kk):
        return zw[k] - zw[kk - 1]

    def z2dzg(k, kk):
        return -zw[k] * zw[k] + zw[kk - 1] * zw[kk - 1]

    def rdzg(k, kk):
        return 1.0 / dzg(k, kk) if k != kk - 1 else 1.0e10
    return dzg, z2dzg, rdzg


def _kraus_turner_col(m, p, tv, k1, pebuoy, ketau):
    """krausturner (goldstein.f90:3337-3442) on one column; tv[k, l] is modified in place.
    Returns (mld, mldk) or None where the routine leaves them untouched."""
    maxk = m.maxk
    ec, ieos, zw, dz = p.ec, p.ieos, m.zw, m.dz
    dec, decd = m.mlddec, m.mlddecd          # [k-1] holds level k
    dzg, z2dzg, rdzg = _level_pair_grids(zw)
    top = maxk                               # mldpk, reset to maxk by the routine
    k = top
    empe = pebuoy
    emke = ketau * dec[k - 1]
    em = empe + emke
    eneed = 0.0
    tmix, smix = tv[k, 0], tv[k, 1]
    q = tv[k, :].copy()
    rhomix = eos(ec, tmix, smix, zw[k], ieos)
    rhou = rhol = 0.0
    out = None
    partial = True
    while eneed < em and em > 0:
        if k < top:
            q[0], q[1] = tmix, smix
            q[2:] = rdzg(maxk, k) * (q[2:] * dzg(maxk, k + 1) + tv[k, 2:] * dz[k - 1])
        if k == k1:
            out = (zw[k - 1], k)
            partial = False
            em = -1.0e-8
            if k < maxk:
                tv[k:maxk + 1, :] = q[None, :]
            continue
        k -= 1
        emr = (em - eneed) / em
        empe = empe * emr
        emke = emke * emr * decd[k - 1]
        em = empe + emke
        rhou = eos(ec, tmix, smix, zw[k], ieos) if ieos != 0 else rhomix
        tmix = rdzg(maxk, k) * (tmix * dzg(maxk, k + 1) + tv[k, 0] * dz[k - 1])
        smix = rdzg(maxk, k) * (smix * dzg(maxk, k + 1) + tv[k, 1] * dz[k - 1])
        rhol = eos(ec, tv[k, 0], tv[k, 1], zw[k], ieos)
        rhomix = eos(ec, tmix, smix, zw[k], ieos)
        eneed = z2dzg(maxk, k + 1) * rhou + z2dzg(k, k) * rhol - z2dzg(maxk, k) * rhomix
    if partial and em > 0:
        a = dzg(maxk, k + 1) * rdzg(maxk, k) * em / eneed
        b = (dzg(maxk, k) * rdzg(maxk, k + 1) - 1) * a
        below = tv[k, :].copy()
        surf = (1 - b) * q + b * below
        tv[maxk, :] = surf
        if k + 1 <= maxk - 1:
            tv[k + 1:maxk, :] = surf[None, :]
        tv[k, :] = a * q + (1 - a) * below
        out = (zw[k] + em / (zw[k] * (rhol - rhou)) if k < maxk else 0.0, k)
    elif partial and k < maxk:
        out = (zw[k], k + 1)
    return out


def mixed_layer(m, p, ts, ts_before, pe1, mld, mldk):
    """The imld = 1 part of tstepo after co (goldstein.f90:2336-2389): potential energy
    released by co, wind energy, krausturner or the shallow-layer diagnostic."""
    maxi, maxj, maxk = m.maxi, m.maxj, m.maxk
    ec, ieos, zro, zw = p.ec, p.ieos, m.zro, m.zw
    _, z2dzg, _ = _level_pair_grids(zw)
    for i in range(1, maxi + 1):
        for j in range(1, maxj + 1):
            k1 = int(m.k1[j, i])
            if k1 > maxk:
                continue
            pec = 0.0
            for k in range(maxk, 0, -1):
                ro = eos(ec, ts_before[k, j, i, 0], ts_before[k, j, i, 1], zro[k - 1], ieos)
                rn = eos(ec, ts[k, j, i, 0], ts[k, j, i, 1], zro[k - 1], ieos)
                pec = pec + (rn - ro) * z2dzg(k, k)
            peb = pec + pe1[j - 1, i - 1]
            if peb > 0.0:
                peb = peb * p.mldpebuoycoeff
            ketau = m.mldketau[j - 1, i - 1]
            emix = peb + ketau * m.mlddec[maxk - 1]
            if emix > 0.0:
                r = _kraus_turner_col(m, p, ts[:, j, i, :], k1, peb, ketau)
                if r is not None:
                    mld[j - 1, i - 1], mldk[j - 1, i - 1] = r
            else:
                mldk[j - 1, i - 1] = maxk
                p1 = pe1[j - 1, i - 1]
                mld[j - 1, i - 1] = zw[maxk - 1] * (1 - emix / p1) if p1 < 0 else zw[maxk - 1]


def surface_layer_energy(m, p, ts, rho):
    """mldpelayer1 of goldstein.f90:2294-2309, before the flux step: (maxj, maxi)."""
    maxi, maxj, maxk = m.maxi, m.maxj, m.maxk
    _, z2dzg, _ = _level_pair_grids(m.zw)
    t = ts[maxk, 1:maxj + 1, 1:maxi + 1, 0] - ts[maxk + 1, 1:maxj + 1, 1:maxi + 1, 0]
    s = ts[maxk, 1:maxj + 1, 1:maxi + 1, 1] - ts[maxk + 1, 1:maxj + 1, 1:maxi + 1, 1]
    r = eos(p.ec, t, s, m.zro[maxk - 1], p.ieos)
    return (r - rho[maxk, 1:maxj + 1, 1:maxi + 1]) * z2dzg(maxk, maxk)


def tstepo(m, p, ts, ts1, rho, u, cost, icosd, nsteps=1, mld=None, mldk=None):
    """tstepo (goldstein.f90:2280-2432).  In place; returns (dmax, limps) of the last step.
    With p.imld = 1 the mixed-layer diagnostics go to mld, mldk ((maxj, maxi))."""
    maxi, maxj, maxk = m.maxi, m.maxj, m.maxk
    dmax, limps = 0.0, 0
    k1 = m.k1
    for _ in range(nsteps):
        if p.imld == 1:
            pe1 = surface_layer_energy(m, p, ts, rho)
        dmax, limps = flux(m, p, ts, ts1, rho, u)
        if p.imld == 1:
            before = ts[..., :2].copy()
            co(m, p, ts, rho, cost, icosd)
            mixed_layer(m, p, ts, before, pe1, mld, mldk)
        else:
            co(m, p, ts, rho, cost, icosd)
        if p.ieos:
            wet = k1[1:maxj + 1, 1:maxi + 1] <= maxk
            t = ts[1:maxk + 1, 1:maxj + 1, 1:maxi + 1]
            r = eos(p.ec, t[..., 0], t[..., 1], m.zro[:, None, None], p.ieos)
            rho[1:maxk + 1, 1:maxj + 1, 1:maxi + 1] = np.where(wet[None], r, rho[1:maxk + 1, 1:maxj + 1, 1:maxi + 1])
        for j in range(1, maxj + 1):
            for k in range(int(k1[j, 0]), maxk + 1):
                rho[k, j, 0] = rho[k, j, maxi]
                ts1[k, j, 0] = ts[k, j, maxi]
            for k in range(int(k1[j, maxi + 1]), maxk + 1):
                rho[k, j, maxi + 1] = rho[k, j, 1]
                ts1[k, j, maxi + 1] = ts[k, j, 1]
        kk = np.arange(1, maxk + 1)[:, None, None]
        wet3 = kk >= k1[None, 1:maxj + 1, 1:maxi + 1]
        ts1[1:maxk + 1, 1:maxj + 1, 1:maxi + 1] = np.where(
            wet3[..., None], ts[1:maxk + 1, 1:maxj + 1, 1:maxi + 1], ts1[1:maxk + 1, 1:maxj + 1, 1:maxi + 1])
    return dmax, limps
