"""Shared checks for the parity tests (numpy only)."""
import numpy as np

INF_I32 = 1 << 30
MAXV = np.float32(1e8)


def to_ref_float(d):
    """Engine int32 distances -> the reference's float convention."""
    if d.dtype == np.int32:
        out = d.astype(np.float32)
        out[d >= INF_I32] = MAXV
        return out
    return d


def min_weight_matrix(n, ro, col, w):
    """Dense n x n lightest-edge matrix (inf where no edge)."""
    W = np.full((n, n), np.inf, np.float64)
    rows = np.repeat(np.arange(n), np.diff(ro))
    np.minimum.at(W, (rows, col), w.astype(np.float64))
    return W


def has_parallel_edges(n, ro, col):
    rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(ro))
    key = rows * n + np.asarray(col, np.int64)
    return np.unique(key).shape[0] != key.shape[0]


def check_pred_tight(D, P, row_vertex, n, ro, col, w, rtol=0.0, unreached=MAXV):
    """Every finite (s, v) with v != s has a predecessor u such that an edge
    u->v exists and D[s][u] + w(u, v) == D[s][v] (within rtol) for one of the
    parallel u->v entries; unreached entries have predecessor -1;
    P[s][s] == s."""
    D = np.asarray(D, np.float64)
    R = D.shape[0]
    rows = np.arange(R)
    s = np.asarray(row_vertex)
    assert np.all(P[rows, s] == s), "pred[s][s] != s"
    assert np.all(D[rows, s] == 0), "dist[s][s] != 0"
    fin = D < float(unreached) / 10
    assert np.all(P[~fin] == -1), "unreached entry with a predecessor"
    mask = fin.copy()
    mask[rows, s] = False
    rr, vv = np.nonzero(mask)
    uu = P[rr, vv]
    assert np.all((uu >= 0) & (uu < n)), "finite entry without a valid predecessor"
    # candidate weights of the u->v entries: lightest and heaviest (a third
    # distinct parallel weight is checked one by one below)
    src = np.repeat(np.arange(n), np.diff(ro))
    Wmin = np.full((n, n), np.inf)
    Wmax = np.full((n, n), -np.inf)
    np.minimum.at(Wmin, (src, col), np.asarray(w, np.float64))
    np.maximum.at(Wmax, (src, col), np.asarray(w, np.float64))
    assert np.all(np.isfinite(Wmin[uu, vv])), "predecessor is not joined to the vertex by an edge"
    rhs = D[rr, vv]
    tol = rtol * np.maximum(1.0, np.abs(rhs))

    def tight(wt):
        return np.abs(D[rr, uu] + wt - rhs) <= tol

    ok = tight(Wmin[uu, vv]) | tight(Wmax[uu, vv])
    for k in np.nonzero(~ok)[0]:
        u, v = uu[k], vv[k]
        es = np.arange(ro[u], ro[u + 1])
        ws = np.asarray(w, np.float64)[es[np.asarray(col)[es] == v]]
        ok[k] = np.any(np.abs(D[rr[k], u] + ws - rhs[k]) <= tol[k])
    assert np.all(ok), f"{int((~ok).sum())} predecessor edges are not tight"
