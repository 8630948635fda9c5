"""The two-phase form of the convective adjustment, emulated on the CPU (no GPU).

k_co_decide runs co (goldstein.f90:2657-2777) on T and S with co's working list held as a
bit mask of the active levels and logs each merge; k_co_mix replays the log on every other
tracer, then fills from the final mask.  This restates that decomposition in Python (IEEE
doubles, the kernels' operation order; exact FP64 densities, which the kernels' double-float
decisions reproduce, as the -m gpu tests check bit for bit) and compares it with the NumPy
oracle's co on random columns: every tracer and the fill count must be equal bit for bit."""
import math

import numpy as np
import pytest

from oracle import goldstein_np as gnp


def eos(ec, t, s):
    return ((ec[0] * t + ec[1] * s) + ec[2] * (t * t)) + ec[3] * ((t * t) * t)


def co_div(a, b):
    """The kernels' merge division: the logged reciprocal with two residual corrections where
    math.fma exists (Python >= 3.13), else the IEEE quotient it equals (test_division_cpu.py)."""
    if not hasattr(math, "fma"):
        return a / b
    y = 1.0 / b
    q1 = math.fma(math.fma(-b, a * y, a), y, a * y)
    return math.fma(math.fma(-b, q1, a), y, q1)


def decide(ec, dz, tv, k1, maxk):
    """Phase one on T and S (tv[:, 0:2] updated in place): returns (log, final mask, filled)."""
    mask = sum(1 << (lev - 1) for lev in range(k1, maxk + 1))
    dzm = {lev: dz[lev] for lev in range(k1, maxk + 1)}
    rho = {lev: eos(ec, tv[lev, 0], tv[lev, 1]) for lev in range(k1, maxk + 1)}

    def below(x):
        m = mask & ((1 << (x - 1)) - 1)
        return m.bit_length() if m else 0

    def above(x):
        m = mask & ~((1 << x) - 1)
        return (m & -m).bit_length()

    def stable(a, b):
        return rho[a] < rho[b]

    log = []
    x, lastmix = maxk, 0
    while True:
        b = below(x)
        if not (b > 0 or (lastmix and x != maxk)):
            break
        if b <= 0 or stable(x, b):
            x = b if (lastmix == 0 or x == maxk) else above(x)
            lastmix = 0
            continue
        nl = b
        while True:
            bb = below(nl)
            if bb <= 0 or stable(nl, bb):
                break
            nl = bb
        # merge: level x, then the active levels below it down to nl, in co's order
        stretch = [lev for lev in range(x - 1, nl - 1, -1) if mask >> (lev - 1) & 1]
        dtop = dzm[x]
        at, as_, dtot = tv[x, 0] * dtop, tv[x, 1] * dtop, dtop
        parts = []
        for lev in stretch:
            d = dzm[lev]
            dtot = dtot + d
            at = at + tv[lev, 0] * d
            as_ = as_ + tv[lev, 1] * d
            parts.append((lev, d))
        tv[x, 0], tv[x, 1] = co_div(at, dtot), co_div(as_, dtot)
        dzm[x] = dtot
        rho[x] = eos(ec, tv[x, 0], tv[x, 1])
        for lev in stretch:
            mask &= ~(1 << (lev - 1))
        log.append((x, dtop, parts, dtot))
        lastmix = 1
    filled = fill(tv[:, 0:2], mask, k1, maxk)
    return log, mask, filled


def fill(col, mask, k1, maxk):
    n = 0
    for lev in range(k1, maxk):
        if not mask >> (lev - 1) & 1:
            src = ((mask >> lev) & -(mask >> lev)).bit_length() + lev
            col[lev] = col[src]
            n += 1
    return n


def replay(col, log, mask, k1, maxk):
    """Phase two on one tracer's column (in place)."""
    for x, dtop, parts, dtot in log:
        acc = col[x] * dtop
        for lev, d in parts:
            acc = acc + col[lev] * d
        col[x] = co_div(acc, dtot)
    fill(col, mask, k1, maxk)


class _M:
    pass


@pytest.mark.parametrize("seed", range(6))
def test_two_phase_equals_co(seed):
    rng = np.random.default_rng(seed)
    maxk = int(rng.choice([8, 16, 32]))
    L = int(rng.integers(2, 9))
    ec = np.array([-0.0559, 0.7968, -0.0063, 3.7315e-5, 0.0])
    m = _M()
    m.maxk = maxk
    m.dz = rng.uniform(0.02, 0.3, maxk)
    m.zw = np.concatenate([[0.0], np.cumsum(m.dz)])
    p = _M()
    p.ec, p.ieos = ec, 0
    dz = np.concatenate([[0.0], m.dz])
    merges, longest = 0, 0
    for col_n in range(40):
        k1 = int(rng.integers(1, maxk + 1))
        tv = np.zeros((maxk + 2, L))
        kind = col_n % 4
        n = maxk - k1 + 1
        if kind == 0:      # random, mostly unstable
            tv[k1:maxk + 1, 0] = rng.uniform(0.0, 25.0, n)
            tv[k1:maxk + 1, 1] = rng.uniform(-2.0, 2.0, n)
        elif kind == 1:    # exact ties
            tv[k1:maxk + 1, 0] = rng.uniform(0.0, 25.0)
            tv[k1:maxk + 1, 1] = rng.uniform(-2.0, 2.0)
        elif kind == 2:    # stable except near the surface
            tv[k1:maxk + 1, 0] = np.sort(rng.uniform(0.0, 25.0, n))
            tv[maxk, 0] = tv[k1, 0] - 1.0
            tv[k1:maxk + 1, 1] = 0.3
        else:              # alternating
            tv[k1:maxk + 1, 0] = np.where(np.arange(n) % 2 == 0, 5.0, 15.0) + rng.uniform(0, 1e-3, n)
            tv[k1:maxk + 1, 1] = rng.uniform(-0.1, 0.1, n)
        tv[k1:maxk + 1, 2:] = rng.uniform(0.1, 3.0, (n, L - 2))
        ref = tv.copy()
        r = np.zeros(maxk + 1)
        r[1:] = [eos(ec, ref[k, 0], ref[k, 1]) for k in range(1, maxk + 1)]
        filled_ref = gnp._co_col(m, p, ref, r, k1)
        got = tv.copy()
        log, mask, filled = decide(ec, dz, got, k1, maxk)
        for l in range(2, L):
            replay(got[:, l], log, mask, k1, maxk)
        assert filled == filled_ref
        assert np.array_equal(got.view(np.int64), ref.view(np.int64)), (seed, col_n)
        merges += len(log)
        longest = max(longest, len(log))
    # the columns do convect, several times over
    assert merges > 40 and longest >= 3
