"""Node coordinates for generalized (curvilinear) grids.

fst_set_grid takes the nodes of a structured grid, (ni, nj, nk, 3) doubles in
LayoutLeft order with ni = nci + 1 (the reference's `grid` view, filled by
its deck's ``fiesta.initialize_grid``).  ``wavy_box`` builds a smoothly
distorted box, the kind of grid the reference's generalized sample uses (a
sine-perturbed channel); decks with their own ``initialize_grid`` go through
``fiesta_gb300.deck.Deck.grid_nodes``.
"""
import numpy as np


def wavy_box(cfg, amp=0.2, L=1.0):
    """Nodes of a domain of size L per axis whose uniform nodes are displaced
    by up to ``amp`` cell widths along every axis (a positive Jacobian
    everywhere for amp < 0.3)."""
    ni, nj, nk = cfg.nci + 1, cfg.ncj + 1, (cfg.nck + 1 if cfg.ndim == 3 else 1)
    i, j, k = np.meshgrid(np.arange(ni), np.arange(nj), np.arange(nk), indexing="ij")
    h = [L / cfg.nci, L / cfg.ncj, L / cfg.nck if cfg.ndim == 3 else 0.0]
    u, v, w = i / cfg.nci, j / cfg.ncj, (k / cfg.nck if cfg.ndim == 3 else 0.0 * k)
    tp = 2.0 * np.pi
    X = np.zeros((ni, nj, nk, 3), dtype=np.float64, order="F")
    X[..., 0] = L * u + amp * h[0] * np.sin(tp * v + 0.3) * np.cos(tp * w)
    X[..., 1] = L * v + amp * h[1] * np.sin(tp * u + 1.1) * np.cos(tp * w + 0.2)
    if cfg.ndim == 3:
        X[..., 2] = L * w + amp * h[2] * np.sin(tp * u + 0.7) * np.sin(tp * v + 0.4)
    return np.asfortranarray(X)


def terrain_nodes(cfg, height, tdx, tdy, top):
    """Nodes of a terrain-following grid (fiesta.grid.type = "terrain"), as
    readTerrain builds them (src/reader.cpp:121-160): x = tdx*i, y = tdy*j and
    z = h + dz*k with dz = (top - h)/nck, for the ground height h(i, j) given
    at the (nci+1) x (ncj+1) nodes (the restart file's "Height" dataset).
    `tdx`, `tdy`, `top` are the deck's fiesta.tdx, fiesta.tdy, fiesta.h."""
    if cfg.ndim != 3:
        raise ValueError("terrain grids are 3D")
    ni, nj, nk = cfg.nci + 1, cfg.ncj + 1, cfg.nck + 1
    h = np.asarray(height, dtype=np.float64)
    if h.shape != (ni, nj):
        raise ValueError(f"height shape {h.shape} != {(ni, nj)}")
    X = np.zeros((ni, nj, nk, 3), dtype=np.float64, order="F")
    i = np.arange(ni, dtype=np.float64)[:, None, None]
    j = np.arange(nj, dtype=np.float64)[None, :, None]
    k = np.arange(nk, dtype=np.float64)[None, None, :]
    X[..., 0] = tdx * i
    X[..., 1] = tdy * j
    dz = (top - h) / cfg.nck
    X[..., 2] = h[:, :, None] + dz[:, :, None] * k
    return np.asfortranarray(X)
