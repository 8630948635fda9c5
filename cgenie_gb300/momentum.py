"""Device-resident GOLDSTEIN momentum step (include/gb_momentum.h): wind, jbar, the
barotropic streamfunction, the island corrections and velc of step_goldstein
(src/goldstein/goldstein.f90:198-233), reading an FP64 :class:`Goldstein` handle's density and
writing its velocities.

:func:`make_case` builds the momentum inputs of a member with the reference's formulas
(depths and their reciprocals :1360-1384, ku :1386-1391, drag by drgset :2845-2885 with the
namelist's drag, rtv/rtv3 :1409-1415, mk :1459-1474, getj :1486-1495), the psi-point landmass
labels of a .psiles file and an island path per island, for members built with
``MemberConfig(mask="basin")`` or ``"basin_island"`` (the southern boundary and the optional
rectangular island are the islands).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import grid
from .abi import dptr
from .goldstein import GoldsteinError, load_library

FSC = 2 * 7.2921e-5    # Coriolis scale (goldstein_lib.f90:49-52)


class GbMoDims(C.Structure):
    _fields_ = [("maxi", C.c_int32), ("maxj", C.c_int32), ("maxk", C.c_int32), ("isles", C.c_int32),
                ("mpi", C.c_int32), ("solver", C.c_int32)]


class GbMoParams(C.Structure):
    _fields_ = [("dphi", C.c_double), ("rdphi", C.c_double), ("rel", C.c_double)]


_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class GbMoGrid(C.Structure):
    _fields_ = [(n, _dp) for n in ("s", "c", "sv", "cv", "rc", "rcv", "dsv", "rdsv", "ds", "rds", "rds2", "dz", "dza")] + \
               [(n, _ip) for n in ("k1", "ku", "mk", "getj")] + \
               [(n, _dp) for n in ("rh", "drag", "rtv", "rtv3", "psiles")] + \
               [(n, _ip) for n in ("npi", "lpisl", "ipisl", "jpisl")]


def _iptr(a):
    return None if a is None else a.ctypes.data_as(_ip)


@dataclass
class MomentumCase:
    """Momentum inputs of one grid (C-order arrays holding the reference's Fortran layouts)."""
    maxi: int
    maxj: int
    maxk: int
    isles: int
    mpi: int
    dphi: float
    rdphi: float
    rel: float
    arrays: dict
    tau: np.ndarray        # (2, maxi, maxj) as [j, i, l]
    dztau: np.ndarray
    dztav: np.ndarray
    keep: list = field(default_factory=list)

    def dims(self):
        return GbMoDims(self.maxi, self.maxj, self.maxk, self.isles, self.mpi, 0)

    def params(self):
        return GbMoParams(self.dphi, self.rdphi, self.rel)

    def grid(self):
        a = self.arrays
        vals = {}
        for n, t in GbMoGrid._fields_:
            arr = a[n]
            arr = np.ascontiguousarray(arr, dtype=np.int32 if t is _ip else np.float64)
            self.keep.append(arr)
            vals[n] = _iptr(arr) if t is _ip else dptr(arr)
        return GbMoGrid(**vals)


def _labels(dry, maxi, maxj):
    """Connected components (4-neighbour, periodic in i) of the dry psi points dry[j, i-1],
    j = 0..maxj, i = 1..maxi: 1 for the one holding row maxj, 2 for row 0, then 3, 4, ...
    Wet points 0."""
    lab = np.zeros(dry.shape, np.int32)
    nxt = 3
    order = [(maxj, 0), (0, 0)] + [(j, i) for j in range(maxj + 1) for i in range(maxi)]
    for j0, i0 in order:
        if not dry[j0, i0] or lab[j0, i0]:
            continue
        if (j0, i0) == (maxj, 0):
            v = 1
        elif (j0, i0) == (0, 0):
            v = 2
        else:
            v = nxt
            nxt += 1
        stack = [(j0, i0)]
        lab[j0, i0] = v
        while stack:
            j, i = stack.pop()
            for jj, ii in ((j + 1, i), (j - 1, i), (j, (i + 1) % maxi), (j, (i - 1) % maxi)):
                if 0 <= jj <= maxj and dry[jj, ii] and not lab[jj, ii]:
                    lab[jj, ii] = v
                    stack.append((jj, ii))
    return lab


def make_case(member, seed: int = 0, rel: float = 0.9, adrag_days: float = 2.5) -> MomentumCase:
    m = member
    if m.cfg.mask not in ("basin", "basin_island", "file"):
        raise ValueError("momentum cases need a basin mask (MemberConfig(mask='basin' or 'basin_island')) "
                         "or a mask file with its .psiles and .paths")
    rng = np.random.default_rng(seed)
    maxi, maxj, maxk = m.maxi, m.maxj, m.maxk
    hg = grid.horizontal_grid(maxi, maxj)
    k1 = m.k1.T.copy()   # [i, j], 0..maxi+1, 0..maxj+1
    dz = np.asarray(m.dz, float)
    # depths and their reciprocals (goldstein.f90:1360-1384)
    h3 = np.zeros((maxi + 2, maxj + 2))
    rh = np.zeros((3, maxi + 2, maxj + 2))
    for j in range(maxj + 1, -1, -1):
        for i in range(maxi + 2):
            if k1[i, j] <= maxk:
                hh = 0.0
                for k in range(k1[i, j], maxk + 1):
                    hh = hh + dz[k - 1]
                h3[i, j] = hh
                rh[2, i, j] = 1.0 / hh
    for j in range(maxj + 2):
        for i in range(maxi + 1):
            if max(k1[i, j], k1[i + 1, j]) <= maxk:
                rh[0, i, j] = 1.0 / min(h3[i, j], h3[i + 1, j])
    for j in range(maxj + 1):
        for i in range(maxi + 2):
            if max(k1[i, j], k1[i, j + 1]) <= maxk:
                rh[1, i, j] = 1.0 / min(h3[i, j], h3[i, j + 1])
    ku = np.zeros((2, maxi + 1, maxj + 1), np.int32)
    for j in range(1, maxj + 1):
        for i in range(1, maxi + 1):
            ku[0, i, j] = max(k1[i, j], k1[i + 1, j])
            ku[1, i, j] = max(k1[i, j], k1[i, j + 1])
    # drag (drgset, goldstein.f90:2845-2885) with adrag = 1/(adrag_days * 86400 * fsc)
    adrag = 1.0 / (adrag_days * 86400 * FSC)
    drgf, kmxdrg, jeb = 3.0, maxk // 2, 1
    tmp = np.zeros((maxi + 1, maxj + 1))
    for j in range(maxj + 1):
        for i in range(maxi + 1):
            kloc2 = max(k1[i, j], k1[i + 1, j], k1[i, j + 1], k1[i + 1, j + 1])
            kloc4 = k1[i, j]
            for j1 in range(max(0, j - 1), min(maxj + 1, j + 2) + 1):
                for i1 in range(i - 1, i + 3):
                    i1p = 1 + (maxi + i1 - 1) % maxi
                    kloc4 = max(kloc4, k1[i1p, j1])
            if kloc2 > kmxdrg or abs(j - maxj // 2) <= jeb:
                tmp[i, j] = adrag * drgf * drgf
            elif kloc4 > kmxdrg or abs(j - maxj // 2) == jeb + 1:
                tmp[i, j] = adrag * drgf
            else:
                tmp[i, j] = adrag
    drag = np.zeros((2, maxi + 2, maxj + 1))
    for j in range(1, maxj + 1):
        drag[0, 1:maxi + 1, j] = 0.5 * (tmp[1:maxi + 1, j] + tmp[1:maxi + 1, j - 1])
        drag[1, 1:maxi + 1, j] = 0.5 * (tmp[1:maxi + 1, j] + tmp[0:maxi, j])
    drag[1, maxi + 1, :] = drag[1, 1, :]
    s, sv, c, cv = hg["s"], hg["sv"], hg["c"], hg["cv"]
    rtv = np.zeros((maxi + 1, maxj + 1))
    rtv3 = np.zeros((maxi + 1, maxj + 1))
    for j in range(1, maxj + 1):
        for i in range(1, maxi + 1):
            rtv[i, j] = 1.0 / (s[j] * s[j] + drag[0, i, j] * drag[0, i, j])
            rtv3[i, j] = 1.0 / (sv[j] * sv[j] + drag[1, i, j] * drag[1, i, j])
    # mk and getj (goldstein.f90:1459-1495)
    mk = np.zeros((maxi + 2, maxj + 1), np.int32)
    wetf = lambda kk: kk * (1 if maxk - kk >= 0 else 0)   # noqa: E731: k1*(1+SIGN(1,maxk-k1))/2
    for j in range(1, maxj + 1):
        for i in range(1, maxi + 1):
            v = max(wetf(k1[i, j]), wetf(k1[i + 1, j]), wetf(k1[i - 1, j]), wetf(k1[i, j + 1]), wetf(k1[i, j - 1]))
            mk[i, j] = v * (1 if maxk - k1[i, j] >= 0 else 0)
    mk[maxi + 1, 1:maxj + 1] = mk[1, 1:maxj + 1]
    getj = np.zeros((maxi + 1, maxj + 1), np.int32)
    for j in range(1, maxj + 1):
        for i in range(1, maxi + 1):
            getj[i, j] = int(max(k1[i, j], k1[i + 1, j], k1[i, j + 1], k1[i + 1, j + 1]) <= maxk and
                             (k1[i, j] != k1[i, j + 1] or k1[i, j] != k1[i + 1, j] or k1[i, j] != k1[i + 1, j + 1]))
    if m.cfg.mask == "file":
        psiles = grid.read_psiles(m.cfg.mask_file + ".psiles", maxi, maxj)
        isles = int(psiles.max()) - 1
        npi, paths = grid.read_paths(m.cfg.mask_file + ".paths", isles) if isles > 0 else (np.zeros(0, np.int32), [])
        for p in paths:
            for (l_, i_, j_) in p:
                if abs(l_) not in (1, 2) or not (0 <= i_ <= maxi) or not (0 <= j_ <= maxj) or k1[i_, j_] > maxk:
                    raise ValueError(f"bad path point {(l_, i_, j_)}")
        return _case_from(m, rng, hg, dz, k1, ku, mk, getj, rh, drag, rtv, rtv3, psiles, isles, paths, rel)
    # psi-point landmasses (a .psiles file) and the island paths (a .paths file)
    dry = np.zeros((maxj + 1, maxi), bool)
    for j in range(maxj + 1):
        for i in range(1, maxi + 1):
            dry[j, i - 1] = max(k1[i, j], k1[i + 1, j], k1[i, j + 1], k1[i + 1, j + 1]) > maxk
    lab = _labels(dry, maxi, maxj)
    isles = int(lab.max()) - 1
    expect = 2 if m.cfg.mask == "basin_island" else 1
    if isles != expect:
        raise ValueError(f"unexpected landmasses: {isles + 1}")
    psiles = lab.astype(np.float64).reshape(-1)   # index i + j*maxi - 1
    paths = [[(1, i, 1) for i in range(1, maxi + 1)]]   # the southern boundary: eastward along row 1
    if isles == 2:
        (_, _), _, (b0, b1), (c0, c1) = grid.basin_island_cells(maxi, maxj)
        a, b, cc, d = b0 - 1, b1 + 1, c0 - 1, c1 + 1   # the ring of wet cells around the island
        p = [(1, i, cc) for i in range(a, b)] + [(2, b, j) for j in range(cc, d)]
        p += [(-1, i, d) for i in range(b - 1, a - 1, -1)] + [(-2, a, j) for j in range(d - 1, cc - 1, -1)]
        paths.append(p)
    return _case_from(m, rng, hg, dz, k1, ku, mk, getj, rh, drag, rtv, rtv3, psiles, isles, paths, rel)


def _case_from(m, rng, hg, dz, k1, ku, mk, getj, rh, drag, rtv, rtv3, psiles, isles, paths, rel):
    maxi, maxj, maxk = m.maxi, m.maxj, m.maxk
    mpi = max([2 * (maxi + maxj)] + [len(p) for p in paths])
    npi = np.array([len(p) for p in paths], np.int32)
    lp = np.zeros((isles, mpi), np.int32)
    ip = np.zeros((isles, mpi), np.int32)
    jp = np.zeros((isles, mpi), np.int32)
    for n, p in enumerate(paths):
        for q, (l_, i_, j_) in enumerate(p):
            lp[n, q], ip[n, q], jp[n, q] = l_, i_, j_
    # wind stress of the step (goldstein.f90:102-107): dztau, dztav; tau = (dztau(1), dztav(2)) * dzz
    def smooth():
        f = rng.standard_normal((maxj, maxi))
        for _ in range(2):
            f = 0.25 * (np.roll(f, 1, 1) + np.roll(f, -1, 1) + 2 * f)
        return f
    dzz = float(dz[maxk - 1])
    dztau = 0.1 * np.stack([smooth(), smooth()], axis=-1) / dzz
    dztav = 0.1 * np.stack([smooth(), smooth()], axis=-1) / dzz
    tau = np.stack([dztau[..., 0] * dzz, dztav[..., 1] * dzz], axis=-1)
    arrays = dict(
        s=hg["s"], c=hg["c"], sv=hg["sv"], cv=hg["cv"], rc=hg["rc"],
        rcv=1.0 / hg["cv"][1:maxj], dsv=hg["dsv"][:maxj - 1], rdsv=hg["rdsv"][:maxj - 1],
        ds=hg["ds"], rds=hg["rds"],
        rds2=np.array([2.0 / (hg["dsv"][j - 1] + hg["dsv"][j - 2]) for j in range(2, maxj)] or [0.0]),
        dz=dz, dza=np.asarray(m.dza, float)[:maxk],
        k1=m.k1, ku=np.ascontiguousarray(ku[:, 1:, 1:].transpose(2, 1, 0)),
        mk=np.ascontiguousarray(mk[1:, 1:].T), getj=np.ascontiguousarray(getj[1:, 1:].T),
        rh=np.ascontiguousarray(rh.transpose(2, 1, 0)), drag=np.ascontiguousarray(drag[:, 1:, 1:].transpose(2, 1, 0)),
        rtv=np.ascontiguousarray(rtv[1:, 1:].T), rtv3=np.ascontiguousarray(rtv3[1:, 1:].T), psiles=psiles,
        npi=npi, lpisl=lp, ipisl=ip, jpisl=jp)
    return MomentumCase(maxi=maxi, maxj=maxj, maxk=maxk, isles=isles, mpi=mpi, dphi=m.dphi, rdphi=m.rdphi,
                        rel=rel, arrays=arrays, tau=tau, dztau=dztau, dztav=dztav)


class Momentum:
    """A device-resident momentum step (gb_mo handle) for a Goldstein handle of the same grid."""

    def __init__(self, case: MomentumCase, device: int = -1, solver: int = 0):
        """solver: 0 = by grid size (the explicit inverse up to GB_MO_MAX_PSI streamfunction
        points, else the block-tridiagonal solve), 1 = block-tridiagonal at any size."""
        self.lib = load_library()
        self.case = case
        self._dims, self._params, self._grid = case.dims(), case.params(), case.grid()
        self._dims.solver = int(solver)
        h = C.c_void_p()
        rc = self.lib.gb_mo_create(C.addressof(self._dims), C.addressof(self._params), C.addressof(self._grid),
                                   int(device), C.byref(h))
        if rc != 0:
            raise GoldsteinError(rc, "gb_mo_create")
        self.h = h

    def _check(self, rc, what):
        if rc != 0:
            detail = self.lib.gb_mo_last_error(self.h).decode() if self.h else ""
            raise GoldsteinError(rc, what, detail)

    def close(self):
        if self.h:
            self.lib.gb_mo_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_wind(self, tau=None, dztau=None, dztav=None):
        c = self.case
        arrs = [np.ascontiguousarray(c.tau if tau is None else tau, dtype=np.float64),
                np.ascontiguousarray(c.dztau if dztau is None else dztau, dtype=np.float64),
                np.ascontiguousarray(c.dztav if dztav is None else dztav, dtype=np.float64)]
        self._check(self.lib.gb_mo_set_wind(self.h, *[dptr(a) for a in arrs]), "gb_mo_set_wind")

    def step(self, ocean):
        self._check(self.lib.gb_mo_step(self.h, ocean.h), "gb_mo_step")

    def download(self):
        c = self.case
        nu = (c.maxk, c.maxj + 1, c.maxi + 1, 3)
        u, u1 = np.zeros(nu), np.zeros(nu)
        ub = np.zeros((c.maxj + 1, c.maxi + 2, 2))
        psi = np.zeros((c.maxj + 1, c.maxi + 1))
        self._check(self.lib.gb_mo_download(self.h, dptr(u), dptr(u1), dptr(ub), dptr(psi)), "gb_mo_download")
        return dict(u=u, u1=u1, ub=ub, psi=psi)
