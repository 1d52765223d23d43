"""Detector regions of the adjoint response.

The response integrates the absorption rate over a detector given as
per-zone weights det(z), z = (k*ny + j)*nx + i over the whole mesh; a box
detector weighs each zone by the fraction of its volume inside the box, so
the response is the exact integral over the box for zone-wise constant flux.
"""
import numpy as np


def _overlap(edges, lo, hi):
    a, b = edges[:-1], edges[1:]
    return np.clip(np.minimum(b, hi) - np.maximum(a, lo), 0.0, None) / (b - a)


def box_detector(dx, dy, dz, lo, hi, origin=(0.0, 0.0, 0.0)):
    """Zone weights of the box [lo, hi] (cm) on the mesh with spacings dx, dy, dz."""
    fr = []
    for d, o, a, b in zip((dx, dy, dz), origin, lo, hi):
        edges = o + np.concatenate([[0.0], np.cumsum(np.asarray(d, dtype=np.float64))])
        fr.append(_overlap(edges, a, b))
    fx, fy, fz = fr
    return np.einsum("k,j,i->kji", fz, fy, fx).ravel()


def context_box_detector(ctx, lo, hi):
    """box_detector on the mesh of a kripke_gb300 context (the dx/dy/dz fields concatenated over zone sets)."""
    return box_detector(ctx.download("dx"), ctx.download("dy"), ctx.download("dz"), lo, hi)
