"""ORACLE -- test infrastructure only (tests and bench.py's CPU leg use it, the product never does).

Independent NumPy restatement of the reference BIOGEM tracer coupling
(src/biogem/biogem.f90:1885-2077, with the vector form of src/biogem/biogem_lib.f90:1056-1081,
1335-1410), written from the Fortran separately from oracle/biogem_oracle.c so that the two
cross-check each other.  Arrays are NumPy views in Fortran index order:
  go_ts[l, i, j, k]        (n_l_ocn, n_i, n_j, n_k), 0-based
  vocn[n, k, l]            one row per wet column n (i outer, j inner), (n_vocn, n_k, n_l_ocn)
  mass/volume/rmass[n, k]  (n_vocn, n_k)
  vbio_part[n, k, l]       (n_vocn, n_k, n_l_sed)
Fortran's SUM adds left to right from 0: every sum below is an explicit left-to-right
accumulation (`_seqsum`), per column over k from k1, then over the columns in vector order.
"""
import numpy as np

NULLSMALL = 0.999999e-19   # const_real_nullsmall, src/common/gem_cmn.f90:719


def columns(k1, n_k):
    """(i, j, k1) of the wet columns, i outer and j inner (biogem_lib.f90:1069-1079); k1 is (n_i, n_j), 1-based values."""
    n_i, n_j = k1.shape
    return [(i, j, int(k1[i, j])) for i in range(n_i) for j in range(n_j) if n_k >= k1[i, j]]


def _seqsum(x):
    """Left-to-right sum from 0 along the last axis."""
    s = np.zeros(x.shape[:-1])
    for t in range(x.shape[-1]):
        s = s + x[..., t]
    return s


def _colsum(cols, field):
    """Per-column SUM over k = k1..n_k of field[n, k, ...] (0-based k index k1-1..n_k-1)."""
    out = []
    for n, (_, _, kk) in enumerate(cols):
        out.append(_seqsum(np.moveaxis(field[n, kk - 1:], 0, -1)))
    return np.array(out)


def tracercoupling(go_ts, vocn, mass, volume, rmass, vdocn, vbio_part, vdbio_part, k1, ts_offset, force_ts):
    """Returns (go_ts, go_ts1) and updates vocn, mass, rmass, vbio_part in place."""
    L, n_i, n_j, n_k = go_ts.shape
    cols = columns(k1, n_k)
    nv = len(cols)
    wet = np.zeros((nv, n_k), bool)
    vts = np.zeros((nv, n_k, L))
    for n, (i, j, kk) in enumerate(cols):
        wet[n, kk - 1:] = True
        vts[n, kk - 1:, :] = go_ts[:, i, j, kk - 1:].T
    w = wet[..., None]
    off = np.array(ts_offset, float)

    tot_v = _seqsum(_colsum(cols, volume))
    rtot_v = 1.0 / tot_v
    mean_s_old = _seqsum(_colsum(cols, vocn[..., 1] * volume) * rtot_v)
    rmean_s_old = 1.0 / mean_s_old
    tot_old = _seqsum(_colsum(cols, vocn[..., 2:] * mass[..., None]).T) if L > 2 else np.zeros(0)

    loc = np.zeros_like(vts)
    loc[..., :2] = vts[..., :2] + off
    loc[..., 2:] = vts[..., 2:] * vocn[..., 1:2] * rmean_s_old
    loc = np.where(w, loc, 0.0)
    tot_new = _seqsum(_colsum(cols, loc[..., 2:] * mass[..., None]).T) if L > 2 else np.zeros(0)
    rtot_new = np.where(np.abs(tot_new) < NULLSMALL, 0.0, 1.0 / np.where(tot_new == 0.0, 1.0, tot_new))

    ts_new = vts[..., :2] + off + vdocn[..., :2]
    if force_ts:
        loc[..., :2] = np.where(w, ts_new, loc[..., :2])
        vocn[..., :2] = np.where(w, loc[..., :2], vocn[..., :2])
    else:
        vocn[..., :2] = np.where(w, loc[..., :2] + vdocn[..., :2], vocn[..., :2])
    mean_s_new = _seqsum(_colsum(cols, vocn[..., 1] * volume) * rtot_v)
    s_ratio = mean_s_new / mean_s_old
    rs_ratio = 1.0 / s_ratio

    bgc = (tot_old * rtot_new) * loc[..., 2:] + vdocn[..., 2:]
    vocn[..., 2:] = np.where(w, s_ratio * bgc, vocn[..., 2:])
    if vbio_part is not None and vbio_part.shape[-1] > 0:
        vbio_part[...] = np.where(w, s_ratio * (vbio_part + vdbio_part), vbio_part)
    vts_new = np.zeros_like(vts)
    vts_new[..., :2] = loc[..., :2] - off
    with np.errstate(divide="ignore", invalid="ignore"):
        vts_new[..., 2:] = (mean_s_new / vocn[..., 1:2]) * vocn[..., 2:]
    mass[...] = np.where(wet, rs_ratio * mass, mass)
    rmass[...] = np.where(wet, s_ratio * rmass, rmass)

    out = np.zeros_like(go_ts)
    for n, (i, j, kk) in enumerate(cols):
        out[:, i, j, kk - 1:] = vts_new[n, kk - 1:, :].T
    return out, out.copy()
