"""Workflow of the learned stencil classifier: harvest (stencil, TENO cut-off) rows from plain
FP64 solver runs, train the tensor-core MLP on them, and route a mixed-precision solver with it.

The rows come from the reference's own benchmark problems with fresh seeds: the 2D four-quadrant
Riemann problem (TENO5 + HLLC, CFL 0.4) and the 1D Sod tube (TENO5 + HLLC, CFL 0.5), recorded at
several times of each run by the plain solver itself (hteno_harvest)."""
from __future__ import annotations

import numpy as np

from . import ic


def harvest_runs(h, torch, seeds, n=1024, snapshots=(0, 20, 40), keep=0.2, capacity=None,
                 sod_snapshots=(0, 50, 100, 150), device="cuda", shuffle_seed=0):
    """Returns (x int16 [N, 8] BF16 bits, y uint8 [N]) CUDA tensors, shuffled.  The harvest kernels
    append rows in whatever order their threads finish, so the rows are first put in a canonical
    order (sorted by their bits) and then shuffled by a seeded permutation: the same runs give the
    same rows in the same order, and (training being deterministic) the same network."""
    per_2d = (2 * (n + 1) * n) * 8
    if capacity is None:
        capacity = int(len(seeds) * len(snapshots) * per_2d * keep * 1.05) + 8 * 401 * 6 * len(sod_snapshots)
    x = torch.empty((capacity, 8), dtype=torch.int16, device=device)
    y = torch.empty((capacity,), dtype=torch.uint8, device=device)
    off = 0
    for k, seed in enumerate(seeds):
        cfg = h.config(dims=2, nx=n, ny=n, flux=h.FLUX_HLLC, recon=h.RECON_TENO5, precision=h.PREC_FP64)
        with h.Solver(cfg) as s:
            s.set_state(ic.four_quadrant(n, n, seed))
            done = 0
            for snap in snapshots:
                s.step(snap - done)
                done = snap
                got = s.harvest(keep, 1000003 * seed + snap, x[off:], y[off:])
                off = min(capacity, off + got)
    # the 1D benchmark tube: 400 cells, every stencil
    cfg = h.config(dims=1, nx=400, flux=h.FLUX_HLLC, recon=h.RECON_TENO5, cfl=0.5, precision=h.PREC_FP64)
    with h.Solver(cfg) as s:
        s.set_state(ic.sod(400))
        done = 0
        for snap in sod_snapshots:
            s.step(snap - done, 0.2)
            done = snap
            got = s.harvest(1.0, 77 + snap, x[off:], y[off:])
            off = min(capacity, off + got)
    x, y = x[:off].contiguous(), y[:off].contiguous()
    order = canonical_order(torch, x, y)
    gen = torch.Generator(device=device)
    gen.manual_seed(shuffle_seed)
    perm = order[torch.randperm(off, generator=gen, device=device)]
    return x[perm].contiguous(), y[perm].contiguous()


def canonical_order(torch, x, y):
    """Indices that sort rows (x int16 [N, 8], y uint8 [N]) by their bits: x's two 64-bit halves,
    then y (stable sorts from the least significant key), so that the same multiset of rows gives
    the same order however the harvest kernels appended them."""
    order = torch.sort(y.to(torch.int64), stable=True).indices
    keys = x.view(torch.int64)  # the 8 BF16 values of a row as two 64-bit keys
    for k in (1, 0):
        order = order[torch.sort(keys[order, k], stable=True).indices]
    return order


def label_stats(y):
    """Fraction of rows per cut-off pattern (numpy array of 8)."""
    yy = y.cpu().numpy()
    return np.bincount(yy, minlength=8) / max(1, yy.size)


def accuracy(m, torch, x, y, threshold=0.9):
    """(bit accuracy, routed fraction, misroute fraction of routed) of classifier m on rows."""
    p = torch.empty((x.shape[0], 3), dtype=torch.float32, device=x.device)
    m.predict(x, p)
    bits = torch.stack([((y >> k) & 1).bool() for k in range(3)], dim=1)
    acc = ((p > 0.5) == bits).float().mean().item()
    routed = (p > threshold).all(dim=1)
    smooth = y == 7
    nr = routed.sum().item()
    mis = (routed & ~smooth).sum().item()
    return acc, nr / x.shape[0], (mis / nr if nr else 0.0)
