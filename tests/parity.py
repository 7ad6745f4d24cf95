"""Shared helpers for parity tests: relative L2 metrics over whole scenes."""
import numpy as np

FIELDS = ("p0", "px", "py", "vx", "vy")


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    n = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (n if n > 0 else 1.0))


def scene_fields(n_domains, get):
    """Each field concatenated over every domain of the scene."""
    return {f: np.concatenate([np.asarray(get(i, f), dtype=np.float64).ravel() for i in range(n_domains)])
            for f in FIELDS}
