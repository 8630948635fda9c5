"""CPU emulation of the split-precision (FP32-transfer / FP64-state) step, for tests.

It follows the arithmetic of k_step_fp32 without the isoneutral branch:
- per-face transfer coefficients are built in FP64 and kept as an FP32 pair;
- T and S (the density tracers) use FP64 transfers from the pair (the kernel's
  double-float arithmetic agrees with them to ~1e-14);
- other tracers are truncated to FP32 after scaling by 2^s_l, each face
  transfer is evaluated as an FMA of the FP32 coefficients and rounded to int32
  (half to even), and the FP64 state gets T += sum(q) * 2^-s_l / V;
- a tracer whose wet values stay within a factor of two of each other carries an
  offset tref (the mid-range to 8 significant bits): its FP32 value is
  (trunc(T 2^s) - tref 2^s) + trunc(the next 24 bits), and a cell whose signed face
  sums (A + B) do not cancel (D, an FP32 pair) gains rint(tref 2^s * D);
- after every 4th step (steps 0, 4, 8, ... since upload) s_l moves so that
  that step's largest |scaled transfer| of a wet cell would have landed in
  [2^25, 2^26);
- convective adjustment uses the oracle's exact co.

Used to tell the scheme's intrinsic error from kernel defects.
"""
import math

import numpy as np

from cgenie_gb300.abi import GridRefs, dptr, iptr


def trunc32(x):
    f = x.astype(np.float32)
    over = np.abs(f.astype(np.float64)) > np.abs(x)
    f[over] = np.nextafter(f[over], np.float32(0))
    f[np.abs(x) < 2.0 ** -126] = 0.0
    return f


def fma32(a, b, c):
    """float32 fma(a, b, c) (products are exact in float64)."""
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(np.float32)


def coefficients(m):
    """(Ae,Be,An,Bn,Aa,Ba) per interior cell, shape (maxk, maxj, maxi, 6), float32; cmax."""
    maxi, maxj, maxk = m.maxi, m.maxj, m.maxk
    k1 = m.k1
    u = m.u
    d1, d2 = m.diff
    dt = m.dt[0]
    c = np.zeros((maxk, maxj, maxi, 6))
    dsvp = np.zeros(maxj + 1)
    dsvp[1:maxj] = m.dsv[:maxj - 1]
    cv2p = np.zeros(maxj + 2)
    cv2p[1:maxj] = m.cv2[:maxj - 1]
    for k in range(1, maxk + 1):
        for j in range(1, maxj + 1):
            for i in range(1, maxi + 1):
                k1c = k1[j, i]
                ie = 1 if i == maxi else i + 1
                if k >= max(k1c, k1[j, ie]):
                    u1 = u[k - 1, j, i, 0]
                    pec = u1 * m.dphi / d1
                    ups = pec / (2.0 + abs(pec))
                    g = dt * m.ds[j - 1] * m.dz[k - 1]
                    a = u1 * m.rc[j]
                    c[k - 1, j - 1, i - 1, 0] = g * (a * (1.0 - ups) * 0.5 - m.rc2[j] * d1)
                    c[k - 1, j - 1, i - 1, 1] = g * (a * (1.0 + ups) * 0.5 + m.rc2[j] * d1)
                if k >= max(k1c, k1[j + 1, i]):
                    u2 = u[k - 1, j, i, 1]
                    pec = u2 * dsvp[min(j, maxj - 1)] / d1
                    ups = pec / (2.0 + abs(pec))
                    g = dt * m.dphi * m.dz[k - 1]
                    a = m.cv[j] * u2
                    c[k - 1, j - 1, i - 1, 2] = g * (a * (1.0 - ups) * 0.5 - cv2p[j] * d1)
                    c[k - 1, j - 1, i - 1, 3] = g * (a * (1.0 + ups) * 0.5 + cv2p[j] * d1)
                if k1c <= k < maxk:
                    u3 = u[k - 1, j, i, 2]
                    pec = u3 * m.dza[k - 1] / d2
                    ups = pec / (2.0 + abs(pec))
                    g = dt * m.dphi * m.ds[j - 1]
                    c[k - 1, j - 1, i - 1, 4] = g * (u3 * (1.0 - ups) * 0.5 - m.rdza[k - 1] * d2)
                    c[k - 1, j - 1, i - 1, 5] = g * (u3 * (1.0 + ups) * 0.5 + m.rdza[k - 1] * d2)
    c32 = c.astype(np.float32)
    lo = (c - c32.astype(np.float64)).astype(np.float32)
    cmax = float(np.max(np.abs(c32[..., 0::2]).astype(np.float64) + np.abs(c32[..., 1::2])))
    return c32, lo, cmax


def scale_of(g):
    """floor(log2(2^26 / g)) from the exact binary exponent of g, clamped to [-120, 120]."""
    if not (g > 0.0) or not math.isfinite(g):
        return 0
    f, e = math.frexp(g)
    return max(-120, min(120, 26 - e + (1 if f == 0.5 else 0)))


def wet_cells(m):
    kk = np.arange(m.maxk + 2)[:, None, None]
    wet = (kk >= m.k1[None]) & (kk >= 1) & (kk <= m.maxk)
    wet[:, 0] = False
    wet[:, -1] = False
    wet[:, :, 0] = False
    wet[:, :, -1] = False
    return wet


def offsets(m, ts):
    """Per tracer offset tref (float32): the mid-range to 8 significant bits for tracers
    (other than T and S) whose wet values stay within a factor of two of each other."""
    wet = wet_cells(m)
    tref = np.zeros(m.maxl, dtype=np.float32)
    for l in range(2, m.maxl):
        v = ts[..., l][wet]
        lo, hi = float(v.min()), float(v.max())
        if (lo > 0.0 and lo > 0.5 * hi) or (hi < 0.0 and hi < 0.5 * lo):
            f, ex = np.frexp(0.5 * (lo + hi))
            tref[l] = np.float32(np.ldexp(np.rint(f * 256.0), int(ex) - 8))
    return tref


def scales(m, ts, cmax, tref=None, dmax=0.0):
    wet = wet_cells(m)
    out = []
    for l in range(m.maxl):
        off = 0.0 if tref is None else float(tref[l])
        tmax = np.max(np.abs(ts[..., l][wet] - off)) if wet.any() else 0.0
        g = max(2.0 * cmax * tmax, abs(off) * dmax)
        out.append(scale_of(g))
    return out


def divergence_pair(m, c32, lo):
    """Per interior cell the FP32 pair (dh, dl) of D = (Cw - Ce) + (Cs - Cn) + (Cb - Ca),
    C = A + B of a face from the coefficient pairs; zero where |D| <= 2^-40 * sum |C|."""
    maxi = m.maxi
    h = c32.astype(np.float64)
    r = lo.astype(np.float64)
    C = [(h[..., 2 * f] + r[..., 2 * f]) + (h[..., 2 * f + 1] + r[..., 2 * f + 1]) for f in range(3)]
    im = np.r_[maxi, np.arange(1, maxi)] - 1
    cwe = C[0][:, :, im]
    cs = np.zeros_like(C[1])
    cs[:, 1:] = C[1][:, :-1]
    cb = np.zeros_like(C[2])
    cb[1:] = C[2][:-1]
    D = ((cwe - C[0]) + (cs - C[1])) + (cb - C[2])
    S = ((np.abs(cwe) + np.abs(C[0])) + (np.abs(cs) + np.abs(C[1]))) + (np.abs(cb) + np.abs(C[2]))
    keep = np.abs(D) > 2.0 ** -40 * S
    dh = np.where(keep, D, 0.0).astype(np.float32)
    dl = np.where(keep, D - dh.astype(np.float64), 0.0).astype(np.float32)
    return dh, dl


def offset_transfer(tr, dh, dl):
    """rint(tr * (dh + dl)) as the kernel forms it (float32 arrays)."""
    f32 = np.float32
    p = (tr * dh).astype(f32)
    e = (tr.astype(np.float64) * dh.astype(np.float64) - p.astype(np.float64)).astype(f32)
    qi = np.rint(p.astype(np.float64))
    r = ((p - qi.astype(f32)).astype(f32) + (e + (tr * dl).astype(f32)).astype(f32)).astype(f32)
    return (qi + np.rint(r.astype(np.float64))).astype(np.int64)


class Fp32Emulator:
    def __init__(self, m, oracle_mod):
        self.m = m
        self.ts = m.ts.copy()
        self.rho = m.rho.copy()
        self.cost = np.zeros_like(m.cost)
        self.icosd = np.zeros_like(m.icosd)
        self.c, self.clo, self.cmax = coefficients(m)
        self.cd = self.c.astype(np.float64) + self.clo.astype(np.float64)
        self.tref = offsets(m, m.ts)
        self.dh, self.dl = divergence_pair(m, self.c, self.clo)
        dmax = float(np.max(np.abs(self.dh.astype(np.float64)) + np.abs(self.dl.astype(np.float64))))
        self.s = scales(m, m.ts, self.cmax, self.tref, dmax)
        self.oracle = oracle_mod
        self.refs = GridRefs(m)
        rv = np.zeros((m.maxk, m.maxj))
        for k in range(m.maxk):
            for j in range(m.maxj):
                rv[k, j] = 1.0 / (m.dphi * m.ds[j] * m.dz[k])
        self.rv = rv
        self.nstep = 0

    def step(self, n=1):
        import ctypes as C
        m = self.m
        maxi, maxj, maxk, L = m.maxi, m.maxj, m.maxk, m.maxl
        for _ in range(n):
            new = self.ts.copy()
            ip = np.r_[np.arange(2, maxi + 1), 1]
            im = np.r_[maxi, np.arange(1, maxi)]
            for l in range(L):
                sc = 2.0 ** self.s[l]
                if l < 2:
                    T = self.ts[..., l]
                    cfd = self.cd
                    ga_prev = np.zeros((maxj, maxi))
                    for k in range(1, maxk + 1):
                        cf = cfd[k - 1]
                        Tk = T[k]
                        Tc = Tk[1:-1, 1:-1]
                        TE = Tk[1:-1][:, ip]
                        TW = Tk[1:-1][:, im]
                        TN = Tk[2:, 1:-1]
                        TS = Tk[:-2, 1:-1]
                        cw = cf[:, im - 1]
                        cs = np.zeros_like(cf)
                        cs[1:] = cf[:-1]
                        ge = cf[..., 0] * TE + cf[..., 1] * Tc
                        gw = cw[..., 0] * Tc + cw[..., 1] * TW
                        gn = cf[..., 2] * TN + cf[..., 3] * Tc
                        gs = cs[..., 2] * Tc + cs[..., 3] * TS
                        ga = cf[..., 4] * T[k + 1][1:-1, 1:-1] + cf[..., 5] * Tc if k < maxk else np.zeros_like(ge)
                        sm = (gw - ge) + (gs - gn) + (ga_prev - ga)
                        ga_prev = ga
                        wet = k >= m.k1[1:-1, 1:-1]
                        upd = Tc + sm * self.rv[k - 1][:, None]
                        new[k, 1:-1, 1:-1, l] = np.where(wet, upd, Tc)
                    continue
                xs = self.ts[..., l] * sc
                T = trunc32(xs)                            # (maxk+2, maxj+2, maxi+2)
                trs = np.float32(float(self.tref[l]) * sc)
                if trs != 0:
                    lo = trunc32(xs - T.astype(np.float64))
                    T = ((T - trs).astype(np.float32) + lo).astype(np.float32)
                qa_prev = np.zeros((maxj, maxi), dtype=np.int64)
                gmax = np.float32(0.0)
                for k in range(1, maxk + 1):
                    cf = self.c[k - 1]                       # (maxj, maxi, 6)
                    Tk = T[k]
                    Tc = Tk[1:-1, 1:-1]
                    TE = Tk[1:-1][:, ip]
                    TW = Tk[1:-1][:, im]
                    TN = Tk[2:, 1:-1]
                    TS = Tk[:-2, 1:-1]
                    cw = cf[:, im - 1]
                    cs = np.zeros_like(cf)
                    cs[1:] = cf[:-1]
                    ge = fma32(cf[..., 0], TE, (cf[..., 1] * Tc).astype(np.float32))
                    gw = fma32(cw[..., 0], Tc, (cw[..., 1] * TW).astype(np.float32))
                    gn = fma32(cf[..., 2], TN, (cf[..., 3] * Tc).astype(np.float32))
                    gs = fma32(cs[..., 2], Tc, (cs[..., 3] * TS).astype(np.float32))
                    if k < maxk:
                        TU = T[k + 1][1:-1, 1:-1]
                        ga = fma32(cf[..., 4], TU, (cf[..., 5] * Tc).astype(np.float32))
                    else:
                        ga = np.zeros_like(ge)
                    q = [np.rint(g.astype(np.float64)).astype(np.int64) for g in (ge, gw, gn, gs, ga)]
                    sm = (q[1] - q[0]) + (q[3] - q[2]) + (qa_prev - q[4])
                    qa_prev = q[4]
                    wet = k >= m.k1[1:-1, 1:-1]
                    dh, dl = self.dh[k - 1], self.dl[k - 1]
                    if trs != 0 and np.any(dh != 0):
                        qd = offset_transfer(np.full(dh.shape, trs, dtype=np.float32), dh, dl)
                        sm = sm + np.where(dh != 0, qd, 0)
                        if wet.any():
                            gmax = max(gmax, np.abs((trs * dh).astype(np.float32))[wet].max())
                    if wet.any():
                        gm = np.max([np.abs(g)[wet].max() for g in (ge, gw, gn, gs, ga)])
                        gmax = max(gmax, gm)
                    upd = self.ts[k, 1:-1, 1:-1, l] + (sm.astype(np.float64) / sc) * self.rv[k - 1][:, None]
                    new[k, 1:-1, 1:-1, l] = np.where(wet, upd, self.ts[k, 1:-1, 1:-1, l])
                if gmax > 0 and self.nstep % 4 == 0:
                    e = int(np.frexp(np.float32(gmax))[1]) - 1
                    self.s[l] = max(-120, min(120, self.s[l] + 25 - e))
            self.ts = new
            from cgenie_gb300.grid import eos_np
            self.rho[1:maxk + 1] = eos_np(m.ec, new[1:maxk + 1, :, :, 0], new[1:maxk + 1, :, :, 1],
                                          m.zro[:, None, None], m.cfg.ieos)
            r = self.refs
            self.oracle.lib().gbo_co(C.byref(r.dims), C.byref(r.params), C.byref(r.grid), dptr(self.ts),
                                     dptr(self.rho), dptr(self.cost), iptr(self.icosd))
            self.nstep += 1
