"""Shared helpers of the GPU parity tests."""
import numpy as np

from oracle import oracle as O


def pair(shape, L, mu, nu, precision="f64"):
    """(GPU Hooke, oracle Hooke) on the same grid and material."""
    from bri17_gb300 import CartesianGrid, Hooke
    return (Hooke(mu, nu, CartesianGrid(shape, L), precision=precision),
            O.Hooke(mu, nu, O.Grid(shape, L)))


def mean_free_normal(rng, comps, shape):
    u = rng.standard_normal((comps,) + tuple(shape))
    u -= u.reshape(comps, -1).mean(axis=1).reshape((comps,) + (1,) * len(shape))
    return u


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def to_dev(x, dtype=None):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    return t if dtype is None else t.to(dtype)
