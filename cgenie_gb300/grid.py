"""Seeded synthetic GOLDSTEIN members: grid metrics, land mask, velocities, tracers.

The grid follows the reference's own set-up formulas so that every metric the
tracer step reads has the value the model would compute:

* constant-sin(latitude) horizontal grid (``igrid=0``), src/goldstein/goldstein.f90:908-962
* exponential vertical levels with ``ez0=0.1``, goldstein.f90:981-1060
* timestep ``dt = 86400*yearlen/(nyear*tsc)``, goldstein.f90:971-977
* equation-of-state coefficients, goldstein.f90:1063-1075
* nondimensional diffusivities, goldstein.f90:1406-1407
* isoneutral slope limit profile ``ssmax``, goldstein.f90:2057-2070
* vertical velocity from continuity, goldstein.f90:3668-3678
* scales ``usc, rsc, dsc, fsc, rhosc, tsc``, src/goldstein/goldstein_lib.f90:47-54

Arrays are numpy arrays whose C-order memory equals the Fortran column-major
layout of the reference (axes reversed):

* ``ts``/``ts1``: shape ``(maxk+2, maxj+2, maxi+2, maxl)`` = Fortran ``ts(l, 0:maxi+1, 0:maxj+1, 0:maxk+1)``
* ``u``:   shape ``(maxk, maxj+1, maxi+1, 3)`` = Fortran ``u(3, 0:maxi, 0:maxj, 1:maxk)``
* ``rho``: shape ``(maxk+1, maxj+2, maxi+2)`` = Fortran ``rho(0:maxi+1, 0:maxj+1, 0:maxk)``
* ``k1``:  shape ``(maxj+2, maxi+2)`` int32 = Fortran ``k1(0:maxi+1, 0:maxj+1)``
* 1-D metrics are stored from their Fortran lower bound (``rc[0]`` is ``rc(0)``,
  ``cv2[0]`` is ``cv2(1)``, ``dz[0]`` is ``dz(1)``, ``zw[0]`` is ``zw(0)``).

Land is coded as ``k1 = maxk + 1`` by default (any value above ``maxk`` is land,
as in the reference's ``.k1`` files).
"""
from __future__ import annotations

import dataclasses
import math
from typing import Optional

import numpy as np

# goldstein_lib.f90:47-54
PI = math.pi
USC = 0.05
RSC = 6.37e6
DSC = 5.0e3
FSC = 2 * 7.2921e-5
GSC = 9.81
RH0SC = 1.0e3
RHOSC = RH0SC * FSC * USC * RSC / GSC / DSC
TSC = RSC / USC
SALN0 = 34.9


@dataclasses.dataclass
class MemberConfig:
    """One synthetic member.  Physical units as in the namelist (m^2/s, m/s)."""

    maxi: int = 36
    maxj: int = 36
    maxk: int = 16
    maxl: int = 2
    seed: int = 0
    land_frac: float = 0.30
    umax: float = 0.1            # m/s, horizontal velocity magnitude cap
    diff_h: float = 2000.0       # m^2/s  (diff(1))
    diff_v: float = 1.0e-5       # m^2/s  (diff(2))
    nyear: int = 96              # steps per year
    yearlen: float = 365.25
    diso: bool = False
    slope_max: Optional[float] = None   # dimensional isoneutral slope cap; None = namelist ssmax
    ssmaxsurf: float = 10.0      # namelist defaults (goldstein-defaults.nml)
    ssmaxdeep: float = 10.0
    ieos: int = 0
    iconv: int = 0
    iediff: int = 0
    ediff0: float = 0.0          # m^2/s
    ediffpow2: float = 1.0
    tracer_kind: str = "auto"    # "ts": T,S then log-normal; "bgc": T,S,DIC,ALK,PO4,O2,... ; auto
    land_code: int = 0           # 0 -> maxk+1
    forcing: float = 0.0         # amplitude of a seeded surface forcing (0 = none)
    noise: float = 0.5           # degC of seeded T noise (drives convection)
    imld: int = 0                # 1: Kraus-Turner mixed layer (goldstein.f90:2294-2390)
    mldpebuoycoeff: float = 0.15     # namelist default (goldstein-defaults.nml)
    mldwindkedec: float = 25.0       # m, wind-energy decay depth (namelist default)
    mldketau_max: float = 2.0e-5     # seeded stand-in for the wind mixing energy, upper bound
    mask: str = "noise"          # "noise": seeded land fraction; "basin" / "basin_island": one
                                 # continent joined to the north boundary, an open channel in
                                 # rows 1-2 (the southern boundary is an island) and, for
                                 # "basin_island", one rectangular island (momentum tests);
                                 # "file": the .k1 bathymetry at mask_file (read_k1)
    mask_file: str = ""          # mask = "file": path without extension of .k1 (.psiles, .paths)


@dataclasses.dataclass
class Member:
    cfg: MemberConfig
    # dims
    maxi: int
    maxj: int
    maxk: int
    maxl: int
    # params
    diff: np.ndarray
    ec: np.ndarray
    ediff0: float
    ediffpow2: float
    ediffpow2i: int
    # grid metrics
    rc: np.ndarray
    rc2: np.ndarray
    cv: np.ndarray
    cv2: np.ndarray
    dsv: np.ndarray
    rdsv: np.ndarray
    ds: np.ndarray
    rds: np.ndarray
    dz: np.ndarray
    dza: np.ndarray
    rdz: np.ndarray
    rdza: np.ndarray
    zro: np.ndarray
    dt: np.ndarray
    zw: np.ndarray
    ssmax: np.ndarray
    ediff1: np.ndarray
    diffmax: np.ndarray
    k1: np.ndarray
    dphi: float
    rdphi: float
    # state
    ts: np.ndarray
    ts1: np.ndarray
    rho: np.ndarray
    u: np.ndarray
    cost: np.ndarray
    icosd: np.ndarray
    # mixed-layer scheme (read when cfg.imld = 1)
    mlddec: np.ndarray = None        # [1:maxk]
    mlddecd: np.ndarray = None       # [1:maxk]
    mldketau: np.ndarray = None      # (maxj, maxi) = Fortran (1:maxi, 1:maxj)
    mld: np.ndarray = None           # (maxj, maxi) diagnostics
    mldk: np.ndarray = None

    @property
    def wet_cells(self) -> int:
        k1 = self.k1[1:-1, 1:-1]
        wet = k1 <= self.maxk
        return int(np.sum(np.where(wet, self.maxk - k1 + 1, 0)))

    def copy_state(self):
        return (self.ts.copy(), self.ts1.copy(), self.rho.copy(), self.cost.copy(), self.icosd.copy())


def eos_np(ec, t, s, z, ieos):
    """eos, goldstein.f90:3048-3061 (same operation order)."""
    if ieos == 0:
        return ec[0] * t + ec[1] * s + ec[2] * (t * t) + ec[3] * ((t * t) * t)
    return ec[0] * t + ec[1] * s + ec[2] * (t * t) + ec[3] * ((t * t) * t) + ec[4] * t * z


def horizontal_grid(maxi: int, maxj: int):
    """igrid=0 sin-latitude grid, goldstein.f90:908-962."""
    th0, th1 = -PI / 2, PI / 2
    s0, s1 = math.sin(th0), math.sin(th1)
    phix = 2 * PI
    dphi = phix / maxi
    rdphi = 1.0 / dphi
    sv = np.zeros(maxj + 1)
    cv = np.zeros(maxj + 1)
    s = np.zeros(maxj + 1)
    c = np.zeros(maxj + 1)
    sv[0] = s0
    cv[0] = math.cos(th0)
    dscon = (s1 - s0) / maxj
    for j in range(1, maxj + 1):
        sv[j] = s0 + j * dscon
        cv[j] = math.sqrt(max(1 - sv[j] * sv[j], 0.0))
        s[j] = sv[j] - 0.5 * dscon
    ds = np.zeros(maxj)
    rds = np.zeros(maxj)
    rc = np.zeros(maxj + 1)
    rc2 = np.zeros(maxj + 1)
    dsv = np.zeros(max(maxj - 1, 1))
    rdsv = np.zeros(max(maxj - 1, 1))
    cv2 = np.zeros(max(maxj - 1, 1))
    for j in range(1, maxj + 1):
        ds[j - 1] = sv[j] - sv[j - 1]
        rds[j - 1] = 1.0 / ds[j - 1]
        c[j] = math.sqrt(1 - s[j] * s[j])
        rc[j] = 1.0 / c[j]
        rc2[j] = rc[j] * rc[j] * rdphi
        if j < maxj:
            dsv[j - 1] = s[j + 1] - s[j]
            rdsv[j - 1] = 1.0 / dsv[j - 1]
            cv2[j - 1] = cv[j] * cv[j] * rdsv[j - 1]
    return dict(dphi=dphi, rdphi=rdphi, sv=sv, cv=cv, s=s, c=c, ds=ds, rds=rds, rc=rc, rc2=rc2,
                dsv=dsv, rdsv=rdsv, cv2=cv2)


def vertical_grid(maxk: int):
    """Exponential levels (ez0 = 0.1), goldstein.f90:981-1060."""
    ez0 = 0.1
    z1 = ez0 * ((1.0 + 1 / ez0) ** (1.0 / maxk) - 1.0)
    tv4 = ez0 * ((z1 / ez0 + 1) ** 0.5 - 1)
    tv2 = 0.0
    dz = np.zeros(maxk + 1)   # 1-based scratch
    dza = np.zeros(maxk + 1)
    zro = np.zeros(maxk + 1)
    zw = np.zeros(maxk + 1)   # 0-based
    zro[maxk] = -tv4
    zw[maxk] = tv2
    for k in range(1, maxk + 1):
        tv3 = ez0 * ((z1 / ez0 + 1) ** k - 1)
        dz[maxk - k + 1] = tv3 - tv2
        tv2 = tv3
        tv5 = ez0 * ((z1 / ez0 + 1) ** (k + 0.5) - 1)
        if k < maxk:
            dza[maxk - k] = tv5 - tv4
        tv4 = tv5
    for k in range(maxk, 0, -1):
        if k > 1:
            zro[k - 1] = zro[k] - dza[k - 1]
        zw[k - 1] = zw[k] - dz[k]
    rdz = np.zeros(maxk + 1)
    rdza = np.zeros(maxk + 1)
    for k in range(1, maxk):
        rdz[k] = 1.0 / dz[k]
        rdza[k] = 1.0 / dza[k]
    rdz[maxk] = 1.0 / dz[maxk]
    dza[maxk] = 0.0
    return dict(dz=dz[1:].copy(), dza=dza[1:].copy(), rdz=rdz[1:].copy(), rdza=rdza[1:].copy(),
                zro=zro[1:].copy(), zw=zw.copy())


def eos_coefficients(ieos: int) -> np.ndarray:
    """goldstein.f90:1063-1075."""
    ec = np.zeros(5)
    ec[0] = -0.0559 / RHOSC
    ec[1] = 0.7968 / RHOSC
    ec[2] = -0.0063 / RHOSC
    ec[3] = 3.7315e-5 / RHOSC
    ec[4] = 2.5e-5 * DSC / RHOSC if ieos == 1 else 0.0
    return ec


def ssmax_profile(maxk: int, zw: np.ndarray, ssmaxsurf: float, ssmaxdeep: float) -> np.ndarray:
    """goldstein.f90:2057-2070."""
    if -1.0e-7 < ssmaxsurf - ssmaxdeep < 1.0e-7:
        return np.full(maxk - 1, ssmaxdeep)
    mid = 0.5 * (math.log(ssmaxsurf) + math.log(ssmaxdeep))
    dif = 0.5 * (math.log(ssmaxsurf) - math.log(ssmaxdeep))
    efold = 200 / DSC
    dep0 = -300 / DSC
    out = np.zeros(maxk - 1)
    for k in range(1, maxk):
        z = (zw[k] - dep0) / efold
        out[k - 1] = math.exp(mid + dif * math.tanh(z))
    return out


def _smooth_periodic(rng, maxi, maxj, passes=4):
    f = rng.standard_normal((maxj, maxi))
    for _ in range(passes):
        f = (f + np.roll(f, 1, axis=1) + np.roll(f, -1, axis=1)
             + np.vstack([f[:1], f[:-1]]) + np.vstack([f[1:], f[-1:]])) / 5.0
    f -= f.min()
    mx = f.max()
    return f / mx if mx > 0 else f


def make_k1(rng, maxi, maxj, maxk, land_frac, land_code):
    """Seeded land mask + bathymetry, with the reference's halo rules (goldstein.f90:1111-1118)."""
    land = land_code if land_code > maxk else maxk + 1
    passes = max(2, int(round(min(maxi, maxj) / 9)))
    mask_f = _smooth_periodic(rng, maxi, maxj, passes)
    thresh = np.quantile(mask_f, land_frac) if land_frac > 0 else -1.0
    bathy = _smooth_periodic(rng, maxi, maxj, passes)
    nlev = np.clip(np.round(1 + (maxk - 1) * (0.15 + 0.85 * bathy) ** 0.7), 1, maxk).astype(np.int32)
    k1i = (maxk - nlev + 1).astype(np.int32)
    k1i = np.where(mask_f <= thresh, land, k1i).astype(np.int32)
    k1 = np.full((maxj + 2, maxi + 2), land, dtype=np.int32)
    k1[1:maxj + 1, 1:maxi + 1] = k1i
    k1[:, 0] = k1[:, maxi]
    k1[:, maxi + 1] = k1[:, 1]
    k1[0, :] = land
    k1[maxj + 1, :] = land
    return k1


def read_k1(path: str, maxi: int, maxj: int) -> np.ndarray:
    """A .k1 bathymetry file as initialise_goldstein reads it (goldstein.f90:1107-1123):
    rows j = maxj+1 .. 0 of k1(0:maxi+1, j), list-directed; then k1(0,j) = k1(maxi,j) and
    k1(maxi+1,j) = k1(1,j).  Returns k1[j, i], (maxj+2, maxi+2), int32."""
    vals = np.array(open(path).read().split(), dtype=np.int64)
    n = (maxj + 2) * (maxi + 2)
    if vals.size < n:
        raise ValueError(f"{path}: {vals.size} values, {n} expected")
    k1 = np.zeros((maxj + 2, maxi + 2), np.int32)
    for r, j in enumerate(range(maxj + 1, -1, -1)):
        k1[j, :] = vals[r * (maxi + 2):(r + 1) * (maxi + 2)]
        k1[j, 0] = k1[j, maxi]
        k1[j, maxi + 1] = k1[j, 1]
    return k1


def read_psiles(path: str, maxi: int, maxj: int) -> np.ndarray:
    """A .psiles file (goldstein.f90:1502-1518): rows j = maxj .. 0 of the psi-point landmass
    labels, i = 1..maxi; returned as the reference's gbold(i + j*maxi), flat index
    (i - 1) + j*maxi, float64.  isles = its maximum - 1."""
    vals = np.array(open(path).read().split(), dtype=np.float64)
    n = (maxj + 1) * maxi
    if vals.size < n:
        raise ValueError(f"{path}: {vals.size} values, {n} expected")
    out = np.zeros(n)
    for r, j in enumerate(range(maxj, -1, -1)):
        out[j * maxi:(j + 1) * maxi] = vals[r * maxi:(r + 1) * maxi]
    return out


def read_paths(path: str, isles: int):
    """A .paths file (goldstein.f90:1541-1573): npi(1:isles), then per island one skipped
    record and npi(i) records (lpisl, ipisl, jpisl).  Returns (npi, [[(l, i, j), ...], ...])."""
    lines = open(path).read().split("\n")
    tok, r = [], 0
    while len(tok) < isles:
        tok += lines[r].split()
        r += 1
    npi = [int(x) for x in tok[:isles]]
    paths = []
    for n in npi:
        r += 1                       # the record each island's path starts after
        p = []
        for _ in range(n):
            a = lines[r].split()
            p.append((int(a[0]), int(a[1]), int(a[2])))
            r += 1
        paths.append(p)
    return np.array(npi, np.int32), paths


def basin_island_cells(maxi, maxj):
    """(continent i-range, continent first row, island i-range, island j-range), 1-based
    inclusive, of make_k1_basin's layout."""
    w = max(2, maxi // 6)
    ic0 = max(1, maxi // 6)
    jc = max(4, maxj // 3)
    ii0 = ic0 + w + 3
    jj0 = max(4, maxj // 3)
    return (ic0, ic0 + w - 1), jc, (ii0, ii0 + 1), (jj0, jj0 + 1)


def make_k1_basin(rng, maxi, maxj, maxk, land_code, island):
    """Seeded bathymetry on a basin: a continent of columns from row maxj//3 to the north
    boundary, every other cell wet (rows 1-2 always), optionally a 2x2 island with two wet
    cells around it; the reference's halo rules (goldstein.f90:1111-1118)."""
    if maxi < 12 or maxj < 10:
        raise ValueError("basin masks need maxi >= 12 and maxj >= 10")
    land = land_code if land_code > maxk else maxk + 1
    passes = max(2, int(round(min(maxi, maxj) / 9)))
    bathy = _smooth_periodic(rng, maxi, maxj, passes)
    nlev = np.clip(np.round(1 + (maxk - 1) * (0.15 + 0.85 * bathy) ** 0.7), 1, maxk).astype(np.int32)
    k1i = (maxk - nlev + 1).astype(np.int32)
    (a0, a1), jc, (b0, b1), (c0, c1) = basin_island_cells(maxi, maxj)
    k1i[jc - 1:, a0 - 1:a1] = land
    if island:
        k1i[c0 - 1:c1, b0 - 1:b1] = land
    k1 = np.full((maxj + 2, maxi + 2), land, dtype=np.int32)
    k1[1:maxj + 1, 1:maxi + 1] = k1i
    k1[:, 0] = k1[:, maxi]
    k1[:, maxi + 1] = k1[:, 1]
    k1[0, :] = land
    k1[maxj + 1, :] = land
    return k1


def make_velocity(rng, maxi, maxj, maxk, k1, hg, vg, umax):
    """Seeded velocity field u(3,0:maxi,0:maxj,1:maxk), nondimensional.

    Horizontal transport = barotropic part from a streamfunction on psi points
    (zero next to land, so the depth-integrated flow is discretely
    non-divergent) + a baroclinic part whose depth integral over each face
    vanishes.  w is then built from continuity with the reference formula
    (goldstein.f90:3668-3678), so the flow is 3-D non-divergent and w at the
    surface vanishes to rounding.
    """
    dz = vg["dz"]
    c, cv, rds, dphi, rdphi, rc = hg["c"], hg["cv"], hg["rds"], hg["dphi"], hg["rdphi"], hg["rc"]
    u = np.zeros((maxk, maxj + 1, maxi + 1, 3))
    if umax == 0:
        return u
    wet = k1 <= maxk
    # psi on corners (i=0..maxi, j=0..maxj) periodic in i
    psi = np.zeros((maxj + 1, maxi + 1))
    raw = _smooth_periodic(rng, maxi, maxj + 1, 3) - 0.5
    for j in range(maxj + 1):
        for i in range(maxi + 1):
            ii = i if i > 0 else maxi
            ok = (wet[j, ii] and wet[j, ii + 1 if ii < maxi + 1 else ii] and wet[j + 1, ii]
                  and wet[j + 1, ii + 1 if ii < maxi + 1 else ii])
            psi[j, i] = raw[j, (ii - 1) % maxi] if ok else 0.0
    psi[:, 0] = psi[:, maxi]
    # baroclinic profile shape: a few vertical modes
    zr = np.linspace(0, 1, maxk)
    modes = np.stack([np.cos(math.pi * (m + 1) * zr) for m in range(3)])
    u1 = np.zeros((maxk, maxj + 2, maxi + 2))   # east faces (k, j, i), i = 0..maxi
    u2 = np.zeros((maxk, maxj + 2, maxi + 2))   # north faces
    for j in range(1, maxj + 1):
        for i in range(1, maxi + 1):
            # east face of (i, j)
            ip = i + 1
            kf = max(k1[j, i], k1[j, ip])
            if kf <= maxk:
                levs = np.arange(kf, maxk + 1)
                H = dz[levs - 1].sum()
                U = -(psi[j, i] - psi[j - 1, i]) * c[j] * dphi * rds[j - 1]
                prof = (rng.standard_normal(3) @ modes)[levs - 1]
                prof = prof - (prof * dz[levs - 1]).sum() / H
                u1[levs - 1, j, i] = U / H + 0.35 * prof
            # north face of (i, j)
            jp = j + 1
            kf = max(k1[j, i], k1[jp, i])
            if kf <= maxk and j < maxj:
                levs = np.arange(kf, maxk + 1)
                H = dz[levs - 1].sum()
                V = (psi[j, i] - psi[j, i - 1]) / cv[j]
                prof = (rng.standard_normal(3) @ modes)[levs - 1]
                prof = prof - (prof * dz[levs - 1]).sum() / H
                u2[levs - 1, j, i] = V / H + 0.35 * prof
    mx = max(np.abs(u1).max(), np.abs(u2).max())
    scale = (umax / USC) / mx if mx > 0 else 0.0
    u1 *= scale
    u2 *= scale
    u1[:, :, 0] = u1[:, :, maxi]
    u2[:, :, 0] = u2[:, :, maxi]
    u[:, :, :, 0] = u1[:, :maxj + 1, :maxi + 1]
    u[:, :, :, 1] = u2[:, :maxj + 1, :maxi + 1]
    # w from continuity (velc, goldstein.f90:3668-3678)
    for j in range(1, maxj + 1):
        for i in range(1, maxi + 1):
            tv = 0.0
            for k in range(k1[j, i], maxk):
                tv1 = (u[k - 1, j, i, 0] - u[k - 1, j, i - 1, 0]) * rdphi * rc[j]
                tv2 = (u[k - 1, j, i, 1] * cv[j] - u[k - 1, j - 1, i, 1] * cv[j - 1]) * rds[j - 1]
                u[k - 1, j, i, 2] = tv - dz[k - 1] * (tv1 + tv2)
                tv = u[k - 1, j, i, 2]
    return u


def make_tracers(rng, cfg, maxi, maxj, maxk, maxl, k1, vg, hg):
    """T (0-25 degC, decreasing with depth), S (34-36 psu stored as S - saln0), then BGC-like tracers."""
    NI, NJ = maxi + 2, maxj + 2
    ts = np.zeros((maxk + 2, NJ, NI, maxl))
    zro = vg["zro"]
    depth = -zro * DSC                       # metres, positive down, per level 1..maxk
    sfc = 0.25 + 0.75 * _smooth_periodic(rng, maxi, maxj, 3)       # (maxj, maxi)
    prof_t = np.exp(-depth / 1000.0)         # decreasing with depth
    T = 25.0 * sfc[None, :, :] * prof_t[:, None, None]
    T = T + cfg.noise * rng.standard_normal(T.shape)
    T = np.clip(T, 0.0, 25.0)
    Sf = 34.0 + 2.0 * _smooth_periodic(rng, maxi, maxj, 3)
    S = Sf[None, :, :] + 0.05 * rng.standard_normal((maxk, maxj, maxi))
    S = np.clip(S, 34.0, 36.0) - SALN0
    fields = [T, S]
    kind = cfg.tracer_kind
    bgc_ranges = [(2000e-6, 2300e-6), (2200e-6, 2450e-6), (0.0, 3e-6), (0.0, 350e-6)]
    for l in range(2, maxl):
        if kind in ("bgc", "auto") and l - 2 < len(bgc_ranges):
            lo, hi = bgc_ranges[l - 2]
            f = lo + (hi - lo) * (0.5 * _smooth_periodic(rng, maxi, maxj, 3)[None]
                                  + 0.5 * rng.random((maxk, maxj, maxi)))
        else:
            mu = rng.uniform(-14.0, -6.0)
            f = np.exp(mu + 0.5 * rng.standard_normal((maxk, maxj, maxi)))
        fields.append(f)
    k1i = k1[1:maxj + 1, 1:maxi + 1]
    kk = np.arange(1, maxk + 1)[:, None, None]
    wetmask = kk >= k1i[None, :, :]
    for l in range(maxl):
        ts[1:maxk + 1, 1:maxj + 1, 1:maxi + 1, l] = np.where(wetmask, fields[l], 0.0)
    # periodic halos (goldstein.f90:1760-1773)
    ts[:, :, 0, :] = ts[:, :, maxi, :]
    ts[:, :, maxi + 1, :] = ts[:, :, 1, :]
    if cfg.forcing:
        top = cfg.forcing * (2 * rng.random((maxj, maxi, maxl)) - 1) * 1e-3
        ts[maxk + 1, 1:maxj + 1, 1:maxi + 1, :] = np.where((k1i <= maxk)[:, :, None], top, 0.0)
    return ts


def make_member(cfg: MemberConfig) -> Member:
    rng = np.random.default_rng(cfg.seed)
    maxi, maxj, maxk, maxl = cfg.maxi, cfg.maxj, cfg.maxk, cfg.maxl
    hg = horizontal_grid(maxi, maxj)
    vg = vertical_grid(maxk)
    if cfg.mask == "noise":
        k1 = make_k1(rng, maxi, maxj, maxk, cfg.land_frac, cfg.land_code)
    elif cfg.mask == "file":
        k1 = read_k1(cfg.mask_file + ".k1", maxi, maxj)
    else:
        k1 = make_k1_basin(rng, maxi, maxj, maxk, cfg.land_code, island=cfg.mask == "basin_island")
    u = make_velocity(rng, maxi, maxj, maxk, k1, hg, vg, cfg.umax)
    ts = make_tracers(rng, cfg, maxi, maxj, maxk, maxl, k1, vg, hg)
    ec = eos_coefficients(cfg.ieos)
    diff = np.array([cfg.diff_h / (RSC * USC), cfg.diff_v * RSC / (USC * DSC * DSC)])
    tv = 86400.0 * cfg.yearlen / (cfg.nyear * TSC)
    dt = np.full(maxk, tv)
    if cfg.slope_max is not None:
        ss = (cfg.slope_max * RSC / DSC) ** 2
        ssmax = np.full(maxk - 1, ss)
    else:
        ssmax = ssmax_profile(maxk, vg["zw"], cfg.ssmaxsurf, cfg.ssmaxdeep)
    ediff0 = cfg.ediff0 * RSC / (USC * DSC * DSC)
    if -1e-7 < cfg.ediffpow2 < 1e-7:
        ediffpow2i = 0
    elif 1 - 1e-7 < cfg.ediffpow2 < 1 + 1e-7:
        ediffpow2i = 1
    elif 0.5 - 1e-7 < cfg.ediffpow2 < 0.5 + 1e-7:
        ediffpow2i = 2
    else:
        ediffpow2i = -999
    if cfg.iediff in (1, 2):
        # seeded stand-in for the ediff profile (goldstein.f90:2936-3044): positive, depth dependent
        ediff1 = (diff[1] - ediff0) * (0.5 + rng.random((maxk - 1, maxj, maxi))) * 1e-9
        diffmax = 0.5 * 0.125 * vg["dz"] * vg["dz"] / dt
    else:
        ediff1 = np.zeros((max(maxk - 1, 1), maxj, maxi))
        diffmax = np.zeros(maxk)
    rho = np.zeros((maxk + 1, maxj + 2, maxi + 2))
    rho[1:, :, :] = eos_np(ec, ts[1:maxk + 1, :, :, 0], ts[1:maxk + 1, :, :, 1], vg["zro"][:, None, None], cfg.ieos)
    rho[0, 1:maxj + 1, 1:maxi + 1] = 0.0
    return Member(
        cfg=cfg, maxi=maxi, maxj=maxj, maxk=maxk, maxl=maxl,
        diff=diff, ec=ec, ediff0=ediff0, ediffpow2=cfg.ediffpow2, ediffpow2i=ediffpow2i,
        rc=hg["rc"], rc2=hg["rc2"], cv=hg["cv"], cv2=hg["cv2"], dsv=hg["dsv"], rdsv=hg["rdsv"],
        ds=hg["ds"], rds=hg["rds"], dz=vg["dz"], dza=vg["dza"], rdz=vg["rdz"], rdza=vg["rdza"],
        zro=vg["zro"], dt=dt, zw=vg["zw"], ssmax=ssmax, ediff1=np.ascontiguousarray(ediff1),
        diffmax=diffmax, k1=k1, dphi=hg["dphi"], rdphi=hg["rdphi"],
        ts=ts, ts1=ts.copy(), rho=rho, u=u,
        cost=np.zeros((maxj, maxi)), icosd=np.zeros((maxj, maxi), dtype=np.int32),
        **mld_fields(cfg, rng, maxi, maxj, vg["zro"]),
    )


def mld_fields(cfg: MemberConfig, rng, maxi: int, maxj: int, zro: np.ndarray) -> dict:
    """Inputs of the mixed-layer scheme: the wind-energy decay mlddec/mlddecd of
    goldstein.f90:1676-1685 (from the namelist depth scale), and a seeded stand-in for the
    wind mixing energy mldketau of goldstein.f90:120-140 (uniform in [0, mldketau_max],
    zonally smooth).  Drawn after every other seeded field, so members without the
    scheme are unchanged."""
    maxk = len(zro)
    dec = cfg.mldwindkedec / DSC
    mlddec = np.exp(zro / dec)
    mlddecd = np.empty(maxk)
    mlddecd[:-1] = mlddec[:-1] / mlddec[1:]
    mlddecd[-1] = mlddec[-1]
    if cfg.imld:
        lat = rng.uniform(0.0, 1.0, maxj)
        mldketau = cfg.mldketau_max * lat[:, None] * rng.uniform(0.5, 1.0, (maxj, maxi))
    else:
        mldketau = np.zeros((maxj, maxi))
    return dict(mlddec=mlddec, mlddecd=mlddecd, mldketau=mldketau, mld=np.zeros((maxj, maxi)),
                mldk=np.zeros((maxj, maxi), dtype=np.int32))


def config_c1(seed: int = 1) -> MemberConfig:
    """36x36x16, T and S, diffusivities 2000 / 1e-5 m^2/s, dt = 1/96 yr, no diso."""
    return MemberConfig(maxi=36, maxj=36, maxk=16, maxl=2, seed=seed, diso=False)


def config_c2(seed: int = 2) -> MemberConfig:
    """36x36x16 with 17 tracers, isoneutral branch on, diff(1)=1000 m^2/s, slope cap 1e-3."""
    return MemberConfig(maxi=36, maxj=36, maxk=16, maxl=17, seed=seed, diso=True,
                        diff_h=1000.0, slope_max=1.0e-3, tracer_kind="bgc")


def config_c5(seed: int = 5, nyear: int = 2400) -> MemberConfig:
    """360x180x32 with 24 tracers, 0.3 m/s velocities, a stable dt (1/nyear yr)."""
    return MemberConfig(maxi=360, maxj=180, maxk=32, maxl=24, seed=seed, diso=True,
                        diff_h=1000.0, slope_max=1.0e-3, umax=0.3, nyear=nyear, tracer_kind="bgc")


def ensemble_configs(n: int = 256, seed: int = 3, lmin: int = 2, lmax: int = 24):
    """Mixed ensemble: grids split evenly among 18x18x16, 36x36x16, 36x36x32;
    tracer counts uniform in [lmin, lmax]; diff(1) log-uniform 500-5000 m^2/s,
    diff(2) log-uniform 1e-6-1e-4 m^2/s; distinct seeded masks and velocities."""
    rng = np.random.default_rng(seed)
    shapes = [(18, 18, 16), (36, 36, 16), (36, 36, 32)]
    out = []
    for m in range(n):
        mi, mj, mk = shapes[m % 3]
        out.append(MemberConfig(
            maxi=mi, maxj=mj, maxk=mk, maxl=int(rng.integers(lmin, lmax + 1)),
            seed=int(rng.integers(0, 2**31 - 1)),
            diff_h=float(math.exp(rng.uniform(math.log(500.0), math.log(5000.0)))),
            diff_v=float(math.exp(rng.uniform(math.log(1e-6), math.log(1e-4)))),
            diso=False, tracer_kind="bgc"))
    return out


def error_sample(cfgs, per_shape: int = 3):
    """Indices of members that a long error check runs: for every grid shape of the list,
    the members with the fewest and the most tracers and one in between (tracer counts
    of the mixed ensemble span 2-24, so the sample holds both ends)."""
    by_shape = {}
    for n, c in enumerate(cfgs):
        by_shape.setdefault((c.maxi, c.maxj, c.maxk), []).append(n)
    out = []
    for shape in sorted(by_shape):
        idx = sorted(by_shape[shape], key=lambda n: (cfgs[n].maxl, n))
        pick = [idx[0], idx[-1], idx[len(idx) // 2]][:per_shape]
        for n in pick:
            if n not in out:
                out.append(n)
    return out

