"""Helpers shared by the GPU parity tests."""
import numpy as np


def rel(a, b):
    a = np.asarray(a).reshape(-1)
    b = np.asarray(b).reshape(-1)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def crandn(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def cart_kloc(imN):
    axes = [np.arange(-n / 2, n / 2) / n for n in imN]
    g = np.meshgrid(*axes, indexing="ij")
    return np.stack([a.reshape(-1, order="F") for a in g], axis=1)
