"""Shared checks: FP64 PCA reference, angles, canonical mesh form."""
import numpy as np


def fp64_pca_normals(points, queries_idx, nbr_idx, flip):
    """Smallest-eigenvector normals in float64 of {q} plus its neighbours
    (the IPCA-exact multiset), flipped toward `flip`."""
    P = points.astype(np.float64)
    out = np.empty((len(queries_idx), 3))
    for r, (qi, nb) in enumerate(zip(queries_idx, nbr_idx)):
        nb = nb[nb != 0xFFFFFFFF]
        S = np.concatenate([P[qi:qi + 1], P[nb.astype(np.int64)]])
        C = np.cov(S.T, bias=True)
        w, V = np.linalg.eigh(C)
        n = V[:, 0]
        if np.dot(n, np.asarray(flip, np.float64) - P[qi]) < 0:
            n = -n
        out[r] = n
    return out


def angle_deg(a, b, unsigned=False):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    a = a / np.maximum(np.linalg.norm(a, axis=1, keepdims=True), 1e-300)
    b = b / np.maximum(np.linalg.norm(b, axis=1, keepdims=True), 1e-300)
    c = np.sum(a * b, axis=1)
    if unsigned:
        c = np.abs(c)
    return np.degrees(np.arccos(np.clip(c, -1, 1)))


def canonical_mesh(vkeys, vpos, faces):
    """Mesh as (sorted vertex keys, positions in that order, sorted faces as
    key-index triples rotated to start at their smallest index)."""
    vkeys = np.asarray(vkeys, np.int64)
    order = np.lexsort((vkeys[:, 3], vkeys[:, 2], vkeys[:, 1], vkeys[:, 0]))
    rank = np.empty(len(order), np.int64)
    rank[order] = np.arange(len(order))
    f = rank[np.asarray(faces, np.int64)]
    # rotate each triangle so its smallest index comes first (keeps orientation)
    m = np.argmin(f, axis=1)
    rows = np.arange(len(f))
    f = np.stack([f[rows, m], f[rows, (m + 1) % 3], f[rows, (m + 2) % 3]], axis=1)
    fo = np.lexsort((f[:, 2], f[:, 1], f[:, 0]))
    return vkeys[order], np.asarray(vpos)[order], f[fo]


def fp64_pca_normals_rows(points, queries_idx, nbr, flip, chunk=200_000):
    """Vectorised fp64_pca_normals for rows of one width: nbr is an (m, k)
    array of neighbour indices (all real).  Returns (normals, relative
    eigengap (l2 - l1) / l3 of each covariance, eigenvalues ascending)."""
    P = np.asarray(points, np.float32)
    flip = np.asarray(flip, np.float64)
    m = len(queries_idx)
    out = np.empty((m, 3))
    gap = np.empty(m)
    for a in range(0, m, chunk):
        qi = np.asarray(queries_idx[a:a + chunk], np.int64)
        nb = np.asarray(nbr[a:a + chunk], np.int64)
        S = np.concatenate([P[qi][:, None, :], P[nb]], axis=1).astype(np.float64)
        S -= S.mean(axis=1, keepdims=True)
        C = np.einsum("mki,mkj->mij", S, S) / S.shape[1]
        w, V = np.linalg.eigh(C)
        n = V[:, :, 0]
        flipdir = flip[None, :] - P[qi].astype(np.float64)
        n = np.where((np.sum(n * flipdir, axis=1) < 0)[:, None], -n, n)
        out[a:a + chunk] = n
        gap[a:a + chunk] = (w[:, 1] - w[:, 0]) / np.maximum(w[:, 2], 1e-300)
    return out, gap
