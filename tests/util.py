"""Helpers shared by the tests: error norms and device round trips."""
import numpy as np

U_FIELDS = ("rho", "m_x", "m_y", "m_z", "E")
B_FIELDS = ("b_x", "b_y", "b_z")


def field_errors(x, ref, nub, vector_floor=True):
    """Per-field ||x - ref||_inf / max(||ref||_inf, floor).

    For the momentum components (1-3 of u) and the three b components the
    floor is the largest magnitude over the whole vector field, so a
    component that is zero or round-off level in the reference (m_x, m_z,
    b_z of an Alfven wave along x) is measured against the wave, not
    against its own noise."""
    x = np.asarray(x, dtype=np.float64).reshape(-1, nub)
    r = np.asarray(ref, dtype=np.float64).reshape(-1, nub)
    out = []
    if nub == 5:
        vec = np.abs(r[:, 1:4]).max() if vector_floor else 0.0
        floors = [0.0, vec, vec, vec, 0.0]
    else:
        vec = np.abs(r).max() if vector_floor else 0.0
        floors = [vec, vec, vec]
    for f in range(nub):
        den = max(np.abs(r[:, f]).max(), floors[f], 1e-30)
        out.append(float(np.abs(x[:, f] - r[:, f]).max() / den))
    return out


def max_err(x, ref, nub):
    return max(field_errors(x, ref, nub))


def bits_equal(a, b):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    return a.dtype == b.dtype and a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))
