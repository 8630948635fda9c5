"""ORACLE -- test infrastructure only (tests and bench.py's CPU leg use it, the product never does).

Independent NumPy restatement of the 2-D surface steppers, written from the Fortran
separately from oracle/surface_oracle.c:
  tstipa    src/embm/embm.f90:2039-2138
  tstipsic  src/goldsteinseaice/gold_seaice.f90:937-1058 (its diagnostics of :1046-1056 in
            seaice_diag)
  step_seaice's post-processing  gold_seaice.f90:599-619 (seaice_post)
  tstepsic  src/goldsteinseaice/gold_seaice.f90:844-929 (as whole-array face fluxes: the
            reference's west/south carries are the east/north fluxes of the neighbours)
Arrays are [j, i] views (C order) of the Fortran (i, j) fields; tq is [j, i, l].  Every cell's
arithmetic is elementwise, so whole-array NumPy expressions evaluate the same IEEE operations
in the same order as the Fortran loops.
"""
import numpy as np


def step(kind, maxk, dt, dphi, rdphi, betaz, betam, diffmod0, ppmin, ppmax, diffsic, tsc,
         rc, cv, dsv, rdsv, rds, diffa, k1, tq, tq1, source, vel, pptn, nsteps=1):
    """kind 0: tstipa, kind 1: tstipsic.  rc, cv (0:maxj); dsv, rdsv (1:maxj-1); rds (1:maxj);
    diffa [j, dir, l]; k1 [0:maxj+1, 0:maxi+1]; tq, tq1, source, vel [j, i, l]; pptn [j, i].
    Updates tq (and tq1 for EMBM) in place."""
    maxj, maxi = tq.shape[:2]
    cimp = 0.5
    J = np.arange(1, maxj + 1)[:, None]
    rcj, cvj, rdsj = rc[1:maxj + 1][:, None], cv[1:maxj + 1][:, None], rds[:, None]
    rdsv_j = np.concatenate([rdsv, [0.0]])[:, None]
    dsv_j = np.concatenate([dsv, [1.0]])[:, None]
    for _ in range(nsteps):
        for l in range(2):
            u1, u2 = vel[..., 0], vel[..., 1]
            with np.errstate(divide="ignore", invalid="ignore"):
                if kind == 0:
                    clamp = np.maximum(0.0, np.minimum(1.0, (pptn - ppmin) / (ppmax - ppmin)))
                    e = betaz[l] * u1 * rcj * 0.5 * rdphi
                    dpp = diffa[:, 0, l][:, None] + float(1 - l) * diffmod0 * clamp
                    tv = rcj * rcj * rdphi * dpp * rdphi
                    pec = betaz[l] * u1 * dphi / dpp
                    ups = pec / (2.0 + np.abs(pec))
                    ciw = e * (1 + ups) + tv
                    cie = e * (1 - ups) - tv
                    n = cvj * betam[l] * u2 * 0.5
                    dpp = diffa[:, 1, l][:, None] + float(1 - l) * diffmod0 * clamp
                    tvn = cvj * cvj * rdsv_j * diffa[:, 1, l][:, None]
                    pec = betam[l] * u2 * dsv_j / dpp
                    upsn = pec / (2.0 + np.abs(pec))
                    last = J == maxj
                    tvn = np.where(last, 0.0, tvn)
                    upsn = np.where(last, 0.0, upsn)
                    cis = n * (1 + upsn) + tvn
                    cin = n * (1 - upsn) - tvn
                else:
                    k1c = k1[1:maxj + 1, 1:maxi + 1]
                    drye = maxk < np.maximum(k1c, k1[1:maxj + 1, 2:maxi + 2])
                    dryn = maxk < np.maximum(k1c, k1[2:maxj + 2, 1:maxi + 1])
                    e = u1 * rcj * 0.5 * rdphi
                    tv = rcj * rcj * rdphi * diffsic * rdphi
                    pec = u1 * dphi / diffsic
                    ups = pec / (2.0 + np.abs(pec))
                    ciw = np.where(drye, 0.0, e * (1 + ups) + tv)
                    cie = np.where(drye, 0.0, e * (1 - ups) - tv)
                    n = cvj * u2 * 0.5
                    tvn = cvj * cvj * rdsv_j * diffsic
                    pec = u2 * dsv_j / diffsic
                    upsn = pec / (2.0 + np.abs(pec))
                    cis = np.where(dryn, 0.0, n * (1 + upsn) + tvn)
                    cin = np.where(dryn, 0.0, n * (1 - upsn) - tvn)
            # west and south neighbours' coefficients: periodic in i, 0 below j = 1
            cie_w = np.roll(cie, 1, axis=1)
            ciw_w = np.roll(ciw, 1, axis=1)
            cin_s = np.vstack([np.zeros((1, maxi)), cin[:-1]])
            cis_s = np.vstack([np.zeros((1, maxi)), cis[:-1]])
            src = -source[..., l] * tsc if kind == 1 else -source[..., l]
            wet = np.ones((maxj, maxi), bool) if kind == 0 else (k1[1:maxj + 1, 1:maxi + 1] <= maxk)
            t, t1 = tq[..., l].copy(), tq1[..., l]
            v2 = None
            for it in range(5):
                if it < 4:
                    v2 = cimp * t + (1.0 - cimp) * t1
                else:
                    v2 = 0.5 * (v2 + cimp * t + (1.0 - cimp) * t1)
                ve, vw = np.roll(v2, -1, axis=1), np.roll(v2, 1, axis=1)
                vn = np.vstack([v2[1:], np.zeros((1, maxi))])
                vs = np.vstack([np.zeros((1, maxi)), v2[:-1]])
                flux = src + cie * ve - ciw_w * vw + (cin * vn - cis_s * vs) * rdsj
                cen = ciw - cie_w + (cis - cin_s) * rdsj
                if it < 4:
                    new = (t1 * (1.0 - (1.0 - cimp) * (dt * cen)) - dt * flux) / (1 + cimp * (dt * cen))
                else:
                    new = t1 - dt * flux - dt * v2 * cen
                t = np.where(wet, new, t)
            tq[..., l] = t
        if kind == 0:
            tq1[...] = tq



def seaice_diag(maxk, dt, tsc, k1, tq, tq1, dtha, variceth, varicedy):
    """The thermal and dynamical parts of the last tstipsic's ice change on the ocean cells
    (gold_seaice.f90:1046-1056): variceth = tsc*dtsic*dtha, varicedy = varice - varice1 -
    variceth; tq (varice after the step), tq1, dtha, variceth, varicedy [j, i, l]; the last two
    are updated in place (other cells keep their values)."""
    maxj, maxi = tq.shape[:2]
    wet = (k1[1:maxj + 1, 1:maxi + 1] <= maxk)[..., None]
    th = tsc * dt * dtha
    variceth[...] = np.where(wet, th, variceth)
    varicedy[...] = np.where(wet, tq - tq1 - th, varicedy)



def seaice_post(maxk, k1, tq, tq1, dtha, rhoio, rhoice, hlf, hmin, rdtdim, m2mm):
    """step_seaice's post-processing of a sea-ice step (gold_seaice.f90:599-619) on the ocean
    cells: tq (varice) and tq1 (varice1) [j, i, l] updated in place; returns (fx_delta,
    fw_delta) [j, i], 0 on land (gold_seaice.f90:578-579)."""
    maxj, maxi = tq.shape[:2]
    wet = k1[1:maxj + 1, 1:maxi + 1] <= maxk
    h = tq[..., 0]
    a = tq[..., 1]
    m = np.where(1.0 < a, 1.0, a)                 # MAX(0.0, MIN(1.0, varice(2)))
    a = np.where(0.0 > m, 0.0, m)
    fw = -(rhoio * dtha[..., 0])
    thin = h < hmin
    fx = np.where(thin, -(((h * rhoice) * hlf) * rdtdim), 0.0)
    fw = np.where(thin, fw + (h * rhoio) * rdtdim, fw)
    h = np.where(thin, 0.0, h)
    a = np.where(thin, 0.0, a)
    new = np.stack([h, a], axis=-1)
    tq[...] = np.where(wet[..., None], new, tq)
    tq1[...] = np.where(wet[..., None], new, tq1)
    return np.where(wet, fx, 0.0), np.where(wet, fw * m2mm, 0.0)


def tstepsic(maxk, dt, rdphi, diffsic, tsc, sica, sich, rc, cv, rdsv, rds, k1, tq, tq1, dtha, vel):
    """The explicit sea-ice step; tq, tq1, dtha, vel [j, i, l]; updates tq on wet cells."""
    maxj, maxi = tq.shape[:2]
    rcj, cvj, rdsj = rc[1:maxj + 1][:, None], cv[1:maxj + 1][:, None], rds[:, None]
    rdsv_j = np.concatenate([rdsv, [0.0]])[:, None]
    k1c = k1[1:maxj + 1, 1:maxi + 1]
    k1e = k1[1:maxj + 1, 2:maxi + 2]
    k1n = k1[2:maxj + 2, 1:maxi + 1]
    u1, u2 = vel[..., 0], vel[..., 1]
    ve = np.roll(tq1, -1, axis=1)                                   # cell i+1 (periodic)
    vn = np.concatenate([tq1[1:], np.zeros((1, maxi, 2))], axis=0)  # cell j+1 (row maxj+1 unused: land)
    # east faces: the receiving cell's ice stops advection
    stop_e = np.where(u1 >= 0.0, (ve[..., 1] > sica) | (ve[..., 0] > sich),
                      (tq1[..., 1] > sica) | (tq1[..., 0] > sich))
    stop_n = np.where(u2 >= 0.0, (vn[..., 1] > sica) | (vn[..., 0] > sich),
                      (tq1[..., 1] > sica) | (tq1[..., 0] > sich))
    fe = np.zeros_like(tq1)
    fn = np.zeros_like(tq1)
    for l in range(2):
        adv = np.where(stop_e, 0.0, u1 * rcj * (ve[..., l] + tq1[..., l]) * 0.5)
        fe[..., l] = np.where(maxk < np.maximum(k1c, k1e), 0.0,
                              adv - (ve[..., l] - tq1[..., l]) * rcj * rcj * rdphi * diffsic)
        adv = np.where(stop_n, 0.0, cvj * u2 * (vn[..., l] + tq1[..., l]) * 0.5)
        fn[..., l] = np.where(maxk < np.maximum(k1c, k1n), 0.0,
                              adv - cvj * cvj * (vn[..., l] - tq1[..., l]) * rdsv_j * diffsic)
    fw = np.roll(fe, 1, axis=1)
    fs = np.concatenate([np.zeros((1, maxi, 2)), fn[:-1]], axis=0)
    new = tq1 - dt * ((fe - fw) * rdphi + (fn - fs) * rdsj[..., None]) + tsc * dt * dtha
    wet = (k1c <= maxk)[..., None]
    tq[...] = np.where(wet, new, tq)
