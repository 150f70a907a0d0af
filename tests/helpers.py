"""Shared helpers for the parity tests (seeded inputs, mesh descriptions)."""
import numpy as np

SINE_OMEGA = 3.0 * np.pi


def splitmix_uniform(n, seed):
    """Counter-based uniform[-1, 1) values: SplitMix64(seed ^ index) -> top 53 bits."""
    idx = np.arange(n, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = (np.uint64(seed) ^ idx) + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    u = (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return 2.0 * u - 1.0


def mesh_kwargs(kind, n=3):
    """Named test meshes (cells per direction n)."""
    if kind == "dirichlet":
        return dict(n_cells=(n, n, n), bc=(0,) * 6)
    if kind == "mixed":  # Dirichlet plus a Neumann side at x=+1 (sine application)
        return dict(n_cells=(n, n + 1, n), lo=(-1, -1, -1), hi=(1, 1, 1), bc=(0, 1, 0, 0, 0, 0))
    if kind == "periodic":
        return dict(n_cells=(n, n, n + 1), periodic=(1, 1, 1))
    if kind == "partial_periodic":
        return dict(n_cells=(n + 1, n, n), periodic=(1, 0, 0), bc=(0, 0, 1, 0, 0, 1))
    if kind == "anisotropic":
        return dict(n_cells=(n, 2, n + 2), lo=(0, 0, 0), hi=(1.0, 0.5, 2.0), bc=(1, 0, 0, 0, 1, 0))
    if kind == "curved":
        return dict(n_cells=(n, n, n), lo=(-1, -1, -1), hi=(1, 1, 1), bc=(0, 1, 0, 0, 0, 0), deform_amp=0.15,
                    deform_freq=2, deform_left=-1.0, deform_right=1.0, mapping_degree=3)
    raise ValueError(kind)
