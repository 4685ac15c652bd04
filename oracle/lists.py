"""Oracle-side helper (test infrastructure): expands per-column candidate
lists into the per-point,
weighted lists the oracle's LETKF takes (the library does this expansion
inside its kernel)."""
from __future__ import annotations

import numpy as np


def gaspari_cohn(z: np.ndarray) -> np.ndarray:
    z = np.abs(np.asarray(z, dtype=np.float64))
    out = np.zeros_like(z)
    a = z <= 1.0
    b = (z > 1.0) & (z < 2.0)
    za = z[a]
    out[a] = (((-0.25 * za + 0.5) * za + 0.625) * za - 5.0 / 3.0) * za * za + 1.0
    zb = z[b]
    out[b] = ((((zb / 12.0 - 0.5) * zb + 0.625) * zb + 5.0 / 3.0) * zb - 5.0) * zb + 4.0 - 2.0 / (3.0 * zb)
    return out


def point_lists(cols, nlev, col_off, col_idx, col_dist, obs_lev, hsupport, vsupport, compat=False):
    """Per-point (col, lev) CSR lists with localisation weights.

    cols: columns to expand (array); returns (points as (col, lev) pairs,
    offsets, idx, weights)."""
    pts, offs, idxs, ws = [], [0], [], []
    for c in cols:
        e0, e1 = int(col_off[c]), int(col_off[c + 1])
        oi = col_idx[e0:e1]
        dh = col_dist[e0:e1] if col_dist is not None else None
        for lev in range(nlev):
            keep = np.ones(e1 - e0, dtype=bool)
            w = np.ones(e1 - e0)
            if obs_lev is not None:
                dl = np.abs(float(lev) - obs_lev[oi])
                keep &= dl <= vsupport
                if not compat:
                    w = w * gaspari_cohn(dl / (0.5 * vsupport))
            if not compat:
                if dh is not None:
                    w = w * gaspari_cohn(dh / (0.5 * hsupport))
                keep &= w > 0
            pts.append((c, lev))
            idxs.append(oi[keep])
            ws.append(w[keep])
            offs.append(offs[-1] + int(keep.sum()))
    return (np.array(pts, dtype=np.int64).reshape(-1, 2), np.array(offs, dtype=np.int64),
            np.concatenate(idxs).astype(np.int32) if idxs else np.zeros(0, np.int32),
            np.concatenate(ws) if ws else np.zeros(0))
